// driver_loop.cu -- the reference driver's GPU update loop (src/main.cpp:225-327,
// 414-415) linked against libpfa_gb300.so through the reference's own C++
// entry points (mangled names, HostData / CudaData), for the drop-in tests.
//
// Compiled two ways:
//   * -DPFA_REF_HEADERS with the reference's src/ on the include path: the
//     caller's own headers (src/data.cuh, src/discretization.cuh, src/type.h);
//     linking proves every entry point resolves with the reference's
//     signatures, and `layout` prints the structure layout they define;
//   * without it, against include/pfa_reference_abi.h (runs on the GPU).
//
//   driver_loop layout
//       offsets and sizes of HostData / CudaData, one "name offset" per line
//   driver_loop run IN OUT STEPS IO PRECISION [NUC_INTERVAL SIGMA UNIT_A DX DT_NUC]
//       IN: int32 nx, ny, then the four *_old fields (x_Cr, x_Nb, phi_del,
//       phi_lav), nx*ny doubles each, ghost ring included, then 14 doubles:
//       dx, dy, kappa[2], omega[2], Lmob[2], D_Cr[2], D_Nb[2], alpha, dt (the
//       mask is five_point_Laplacian_stencil's from dx, dy).  OUT: for every output step
//       (every IO steps, as io_step in src/main.cpp:323) the step index and
//       the six arrays device_dataviz fills (x_Cr, x_Nb, x_Ni, phi_del,
//       phi_lav, phi) followed by the four read_out_result fills.
//       PRECISION 0 = FP64 as the reference; 1 = the FP32 form, selected with
//       pfa_set_precision right after init_cuda.  NUC_INTERVAL > 0 calls
//       device_nucleation after every step k with k % NUC_INTERVAL == 0
//       (src/main.cpp:307-316; fixed geometry, seed 42).
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef PFA_REF_HEADERS
#include "data.cuh"
#include "discretization.cuh"
#else
#include "pfa_reference_abi.h"
#endif
#include "pfa_gb300.h"

namespace {

// Row-pointer arrays over one contiguous block per field (the arrangement of
// make_arrays, src/mesh.cpp:12-97, with ny row pointers per field).
struct HostArrays {
  std::vector<std::vector<double>> blocks;
  std::vector<std::vector<double*>> rows;

  double** field(int nrows, int ncols) {
    blocks.emplace_back(size_t(nrows) * ncols, 0.0);
    rows.emplace_back(nrows);
    for (int j = 0; j < nrows; j++) rows.back()[j] = blocks.back().data() + size_t(j) * ncols;
    return rows.back().data();
  }
};

void make_host(HostData* h, HostArrays& a, int nx, int ny, int nm) {
  h->mask_lap = a.field(nm, nm);
  double*** f[] = {&h->conc_Ni,     &h->phi,         &h->chem_nrg,    &h->grad_nrg,
                   &h->conc_Cr_old, &h->conc_Cr_new, &h->conc_Cr_lap, &h->conc_Cr_gam,
                   &h->conc_Nb_old, &h->conc_Nb_new, &h->conc_Nb_lap, &h->conc_Nb_gam,
                   &h->phi_del_old, &h->phi_del_new, &h->phi_del_lap, &h->phi_lav_old,
                   &h->phi_lav_new, &h->phi_lav_lap};
  for (auto p : f) *p = a.field(ny, nx);
}

// src/mesh.cpp:33-36 (swap_pointers_1D)
void swap_1d(double** a, double** b) {
  double* t = *a;
  *a = *b;
  *b = t;
}

int layout() {
#define H(n) std::printf("HostData.%s %zu\n", #n, offsetof(HostData, n))
#define C(n) std::printf("CudaData.%s %zu\n", #n, offsetof(CudaData, n))
  H(mask_lap); H(conc_Ni); H(phi); H(chem_nrg); H(grad_nrg);
  H(conc_Cr_old); H(conc_Cr_new); H(conc_Cr_lap); H(conc_Cr_gam);
  H(conc_Nb_old); H(conc_Nb_new); H(conc_Nb_lap); H(conc_Nb_gam);
  H(phi_del_old); H(phi_del_new); H(phi_del_lap);
  H(phi_lav_old); H(phi_lav_new); H(phi_lav_lap);
  C(prng); C(str_A); C(str_B); C(str_C); C(str_D); C(ev_A); C(ev_B); C(ev_C); C(ev_D);
  C(conc_Ni); C(phi); C(conc_Cr_old); C(conc_Cr_new); C(conc_Nb_old); C(conc_Nb_new);
  C(phi_del_old); C(phi_del_new); C(phi_lav_old); C(phi_lav_new);
  C(conc_Cr_gam); C(conc_Cr_del); C(conc_Cr_lav); C(conc_Nb_gam); C(conc_Nb_del); C(conc_Nb_lav);
#undef H
#undef C
  std::printf("sizeof.HostData %zu\nsizeof.CudaData %zu\nsizeof.fp_t %zu\n", sizeof(HostData),
              sizeof(CudaData), sizeof(fp_t));
  // the entry points with the caller's signatures (a mismatch fails to compile
  // or, for the mangled names, to link)
  void (*i)(HostData*, const int, const int, const int, const fp_t*, const fp_t*, const fp_t*,
            const fp_t*, const fp_t*, CudaData*) = &init_cuda;
  void (*e)(CudaData*, const int, const int, const int, const int, const int, const fp_t,
            const fp_t) = &device_evolution;
  void (*n)(CudaData*, const int, const int, const int, const int, const int, const fp_t,
            const fp_t, const fp_t, const fp_t, const fp_t, const fp_t, const fp_t,
            const fp_t) = &device_nucleation;
  void (*v)(CudaData*, HostData*, const int, const int, const int, const int, const int) =
      &device_dataviz;
  void (*r)(CudaData*, HostData*, const int, const int) = &read_out_result;
  void (*s[])(CudaData*, const int, const int, const int, const int, const int) = {
      &device_boundaries, &device_fictitious, &fictitious_boundaries,
      &device_laplacian_boundaries, &device_init_prng};
  void (*l)(CudaData*, const int, const int, const int, const int, const int, const fp_t,
            const fp_t) = &device_laplacian;
  void (*fr)(CudaData*) = &free_cuda;
  cudaError_t (*ck)(cudaError_t) = &checkCuda;
  float (*nt)(int, int, int) = &nTiles;
  const bool all = i && e && n && v && r && s[0] && s[4] && l && fr && ck && nt;
  std::printf("entry_points %d\n", all ? 1 : 0);
  return 0;
}

int fail(const char* what) {
  std::fprintf(stderr, "driver_loop: %s (library error %d: %s)\n", what, pfa_last_error(),
               pfa_last_error_message());
  return 1;
}

int run(int argc, char** argv) {
  if (argc < 7) return fail("usage: run IN OUT STEPS IO PRECISION [NUC...]");
  FILE* in = std::fopen(argv[2], "rb");
  if (!in) return fail("cannot open input");
  int32_t dims[2];
  if (std::fread(dims, sizeof(int32_t), 2, in) != 2) return fail("short input");
  const int nx = dims[0], ny = dims[1], nm = 3, bx = 13, by = 13;
  HostData host;
  HostArrays arrays;
  make_host(&host, arrays, nx, ny, nm);
  double** old[4] = {host.conc_Cr_old, host.conc_Nb_old, host.phi_del_old, host.phi_lav_old};
  for (auto f : old)
    if (std::fread(f[0], sizeof(double), size_t(nx) * ny, in) != size_t(nx) * ny)
      return fail("short input");
  // dx, dy, kappa[2], omega[2], Lmob[2], D_Cr[2], D_Nb[2], alpha, dt
  double c[14];
  if (std::fread(c, sizeof(double), 14, in) != 14) return fail("short input");
  std::fclose(in);
  const double dx = c[0], dy = c[1];
  const double *kappa = c + 2, *omega = c + 4, *Lmob = c + 6, *D_Cr = c + 8, *D_Nb = c + 10;
  const double alpha = c[12], dt = c[13];
  // five_point_Laplacian_stencil, src/mesh.cpp:187-196
  host.mask_lap[0][1] = 1. / (dy * dy);
  host.mask_lap[1][0] = 1. / (dx * dx);
  host.mask_lap[1][1] = -2. * (dx * dx + dy * dy) / (dx * dx * dy * dy);
  host.mask_lap[1][2] = 1. / (dx * dx);
  host.mask_lap[2][1] = 1. / (dy * dy);

  const long steps = std::atol(argv[4]), io_interval = std::atol(argv[5]);
  const int precision = std::atoi(argv[6]);
  const long nuc_interval = argc > 7 ? std::atol(argv[7]) : 0;
  const double sigma = argc > 8 ? std::atof(argv[8]) : 0.13;
  const double unit_a = argc > 9 ? std::atof(argv[9]) : 0.352e-9;
  const double ndx = argc > 10 ? std::atof(argv[10]) : dx;
  const double dt_nuc = argc > 11 ? std::atof(argv[11]) : 0.0;
  FILE* out = std::fopen(argv[3], "wb");
  if (!out) return fail("cannot open output");

  CudaData dev;
  init_cuda(&host, nx, ny, nm, kappa, omega, Lmob, D_Cr, D_Nb, &dev);
  if (pfa_last_error()) return fail("init_cuda");
  if (precision && pfa_set_precision(&dev, precision)) return fail("pfa_set_precision");
  if (nuc_interval > 0 && pfa_set_nucleation(&dev, 42, PFA_NUC_FIXED_GEOMETRY))
    return fail("pfa_set_nucleation");
  device_init_prng(&dev, nx, ny, nm, bx, by);

  const size_t n = size_t(nx) * ny;
  for (long k = 0; k < steps; k++) {
    device_boundaries(&dev, nx, ny, nm, bx, by);
    device_fictitious(&dev, nx, ny, nm, bx, by);
    fictitious_boundaries(&dev, nx, ny, nm, bx, by);
    device_laplacian(&dev, nx, ny, nm, bx, by, dx, dy);
    device_laplacian_boundaries(&dev, nx, ny, nm, bx, by);
    device_evolution(&dev, nx, ny, nm, bx, by, alpha, dt);
    if (nuc_interval > 0 && k % nuc_interval == 0)
      device_nucleation(&dev, nx, ny, nm, bx, by, sigma, sigma, unit_a, 0.0, ndx, ndx, 1.0, dt_nuc);
    swap_1d(&dev.conc_Cr_old, &dev.conc_Cr_new);
    swap_1d(&dev.conc_Nb_old, &dev.conc_Nb_new);
    swap_1d(&dev.phi_del_old, &dev.phi_del_new);
    swap_1d(&dev.phi_lav_old, &dev.phi_lav_new);
    if (pfa_last_error()) return fail("step");
    if ((k + 1) % io_interval == 0) {
      device_dataviz(&dev, &host, nx, ny, nm, bx, by);
      double** viz[6] = {host.conc_Cr_new, host.conc_Nb_new, host.conc_Ni,
                         host.phi_del_new, host.phi_lav_new, host.phi};
      const int32_t step = int32_t(k + 1);
      std::fwrite(&step, sizeof(step), 1, out);
      for (auto f : viz) std::fwrite(f[0], sizeof(double), n, out);
      // read_out_result overwrites the same host arrays: clear them first so
      // that the second record shows what read_out_result itself wrote
      double** res[4] = {host.conc_Cr_new, host.conc_Nb_new, host.phi_del_new, host.phi_lav_new};
      for (auto f : res) std::memset(f[0], 0, n * sizeof(double));
      read_out_result(&dev, &host, nx, ny);
      for (auto f : res) std::fwrite(f[0], sizeof(double), n, out);
      if (pfa_last_error()) return fail("output step");
    }
  }
  std::fclose(out);
  free_cuda(&dev);
  if (pfa_last_error()) return fail("free_cuda");
  if (dev.conc_Cr_old || dev.str_A) return fail("free_cuda left pointers in CudaData");
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc >= 2 && !std::strcmp(argv[1], "layout")) return layout();
  if (argc >= 2 && !std::strcmp(argv[1], "run")) return run(argc, argv);
  std::fprintf(stderr, "usage: driver_loop layout | run ...\n");
  return 2;
}
