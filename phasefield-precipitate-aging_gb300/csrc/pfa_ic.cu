// pfa_ic.cu -- initial conditions built on the device from a recipe (sm_103a).
//
// The reference builds its grids on the host (src/alloy625.cpp:170-518) from
// a matrix composition, enriched regions and particles embedded with
// embed_OPC's tanh profile (:262-294, tanh_interp thermo/nucleation.c:12-16).
// pfa_ic_recipe (pfa_gb300.h) describes such a grid; k_ic_fill evaluates it
// for every interior cell and writes the cell and the ghost cells that mirror
// it, so a grid of any size costs one pass over its FP64 fields and no
// host-to-device copy.  Every product and sum is rounded on its own
// (__dmul_rn / __dadd_rn: no contraction into FMAs) so the noise and band
// terms are bit-identical to a plain FP64 evaluation on the host; tanh and
// p(phi) agree to rounding.
#include <cmath>
#include <cstdint>

#include <cstdio>

#include "pfa_device.cuh"
#include "pfa_gb300.h"
#include "pfa_internal.h"
#include "pfa_kernels.h"

namespace pfa {

using namespace dev;

namespace {

constexpr uint32_t kIcStream = 0x49430000u;  // fourth counter word of the noise draws

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// p(phi) = phi^3 (6 phi^2 - 15 phi + 10) (thermo/parabola625.c:11-18)
__device__ __forceinline__ double p_interp(double x) {
  const double x2 = mul(x, x), x3 = mul(x2, x);
  return mul(x3, add(sub(mul(6.0, x2), mul(15.0, x)), 10.0));
}

// value v of interior cell (x, y, z) into f and into every ghost cell whose
// mirror it is (faces, edges, corners), layout (nz+2) x (ny+2) x (nx+2) or
// (ny+2) x (nx+2) when 2D
__device__ void store_mirrored(double* f, const pfa_ic_recipe& r, bool is3d, int x, int y, int z,
                               double v) {
  int xs[3] = {x + 1, 0, 0}, ys[3] = {y + 1, 0, 0}, zs[3] = {z + 1, 0, 0};
  int nx = 1, ny = 1, nz = 1;
  if (x == 0) xs[nx++] = 0;
  if (x == r.nx - 1) xs[nx++] = r.nx + 1;
  if (y == 0) ys[ny++] = 0;
  if (y == r.ny - 1) ys[ny++] = r.ny + 1;
  if (is3d) {
    if (z == 0) zs[nz++] = 0;
    if (z == r.nz - 1) zs[nz++] = r.nz + 1;
  }
  const size_t sx = size_t(r.nx) + 2, sy = size_t(r.ny) + 2;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const size_t plane = is3d ? size_t(zs[k]) * sy * sx : 0;
        f[plane + size_t(ys[j]) * sx + xs[i]] = v;
      }
}

struct IcOut {
  double* f[4];
  double bellA[2];  // profile 1: the amplitudes that give the curve its mean
};

__global__ void __launch_bounds__(256) k_ic_fill(pfa_ic_recipe r, IcOut o, int is3d) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int z = is3d ? int(blockIdx.z) : 0;
  if (x >= r.nx || y >= r.ny) return;
  const unsigned long long cell =
      (unsigned long long)(size_t(z) * r.ny + y) * (unsigned long long)r.nx + x;
  const uint4 w = philox4x32_10(
      make_uint4(uint32_t(cell), uint32_t(cell >> 32), 0u, kIcStream),
      make_uint2(uint32_t(r.seed), uint32_t(r.seed >> 32)));
  double base[2] = {r.matrix[0], r.matrix[1]};
  if (r.profile == 1) {
    const double pos = mul(r.dx, sub(double(x), r.bell_x0));
    for (int k = 0; k < 2; k++) {
      const double t = pos / r.bell_sigma[k];
      const double v = add(mul(o.bellA[k], sub(exp(mul(-0.5, mul(t, t))), 1.0)), r.enrich[k]);
      base[k] = fmin(1.0, fmax(0.0, v));
    }
  }
  // 2u - 1 is exact for u on the 2^-53 grid
  double xcr = add(base[0], mul(r.noise, sub(mul(2.0, u53(w.x, w.y)), 1.0)));
  double xnb = add(base[1], mul(r.noise, sub(mul(2.0, u53(w.z, w.w)), 1.0)));
  const double dcr = sub(r.enrich[0], r.matrix[0]), dnb = sub(r.enrich[1], r.matrix[1]);
  for (int b = 0; b < r.n_bands; b++)
    if (x >= r.band[b][0] && x < r.band[b][1]) {
      xcr = add(xcr, dcr);
      xnb = add(xnb, dnb);
    }
  double ph[2] = {0.0, 0.0};
  const double half_w = 0.5 * r.width;
  const double coord[3] = {double(x), double(y), double(z)};
  const int dims = is3d ? 3 : 2;
  for (int k = 0; k < r.n_particles; k++) {
    const double R = r.radius[k];
    const int pad = r.particle_mode == 1 ? int(R + 4.0 * r.width / r.dx)
                                         : int(ceil(R + 6.0 * half_w / r.dx)) + 1;
    bool in = true;
    double r2 = 0.0;
    for (int d = 0; d < dims; d++) {
      const double c = r.centre[k][d];
      const int fc = int(floor(c));
      const int q = d == 0 ? x : (d == 1 ? y : z);
      if (q < fc - pad || q > fc + pad) in = false;
      const double t = sub(coord[d], c);
      r2 = add(r2, mul(t, t));
    }
    if (!in) continue;
    const double dist = sqrt(r2);
    const double phi = sub(0.5, mul(0.5, tanh(mul(r.dx, sub(dist, R)) / half_w)));
    const double pp = p_interp(phi);
    const double q = sub(1.0, pp);
    const int phase = r.phase[k] == 0 ? 0 : 1;
    constexpr double xdCr = kXe[1][0], xdNb = kXe[1][1], xlCr = kXe[2][0], xlNb = kXe[2][1];
    const double xe_cr = phase == 0 ? xdCr : xlCr, xe_nb = phase == 0 ? xdNb : xlNb;
    xcr = add(mul(pp, xe_cr), mul(q, xcr));
    xnb = add(mul(pp, xe_nb), mul(q, xnb));
    ph[phase] = r.particle_mode == 1 ? phi : fmax(ph[phase], phi);
  }
  const double v[4] = {xcr, xnb, ph[0], ph[1]};
  for (int f = 0; f < 4; f++) store_mirrored(o.f[f], r, is3d, x, y, z, v[f]);
}

}  // namespace

// Validates a recipe: sizes, counts, finite values (message or nullptr).
const char* ic_check(const pfa_ic_recipe* r) {
  if (!r) return "initial condition: null recipe";
  if (r->nx < 1 || r->ny < 1 || r->nz < 0 || r->nz > 65535)
    return "initial condition: grid sizes must be >= 1 (nz <= 65535)";
  if (r->n_bands < 0 || r->n_bands > PFA_IC_MAX_BANDS)
    return "initial condition: band count out of range";
  if (r->n_particles < 0 || r->n_particles > PFA_IC_MAX_PARTICLES)
    return "initial condition: particle count out of range";
  if (!(r->dx > 0) || !(r->width > 0) || !std::isfinite(r->dx) || !std::isfinite(r->width))
    return "initial condition: dx and width must be finite and > 0";
  for (int k = 0; k < r->n_particles; k++) {
    if (!std::isfinite(r->radius[k]) || r->radius[k] < 0 || r->radius[k] > 4096)
      return "initial condition: particle radius must be in [0, 4096] cells";
    for (int d = 0; d < 3; d++)
      if (!std::isfinite(r->centre[k][d]) || std::fabs(r->centre[k][d]) > 1e9)
        return "initial condition: particle centre not finite";
  }
  // the box pad (radius + three or four widths) stays an int
  if (r->n_particles > 0 && !(4.0 * r->width / r->dx < 1e6))
    return "initial condition: interface width above 1e6 cells";
  if (r->profile != 0 && r->profile != 1) return "initial condition: profile must be 0 or 1";
  if (r->particle_mode != 0 && r->particle_mode != 1)
    return "initial condition: particle_mode must be 0 or 1";
  if (r->profile == 1) {
    for (int k = 0; k < 2; k++)
      if (!(r->bell_sigma[k] > 0) || !std::isfinite(r->bell_sigma[k]))
        return "initial condition: bell widths must be finite and > 0";
    if (!(r->bell_range[1] > r->bell_range[0]) || !std::isfinite(r->bell_range[0]) ||
        !std::isfinite(r->bell_range[1]) || !std::isfinite(r->bell_x0))
      return "initial condition: bell range must be finite with a < b";
  }
  return nullptr;
}

// amplitude of the bell curve whose mean over [a, b] is x0 (thermo/enrichment.py:
// mean of A (exp(-x^2/(2 s^2)) - 1) + xe over [a, b] = A (I / (b - a) - 1) + xe,
// I = s sqrt(pi/2) (erf(b / (s sqrt 2)) - erf(a / (s sqrt 2))))
double ic_bell_amplitude(double sigma, double a, double b, double x0, double xe) {
  const double I = sigma * std::sqrt(M_PI / 2.0) *
                   (std::erf(b / (sigma * std::sqrt(2.0))) - std::erf(a / (sigma * std::sqrt(2.0))));
  return (x0 - xe) / (I / (b - a) - 1.0);
}

cudaError_t launch_ic_fill(const pfa_ic_recipe& r, double* const f[4], cudaStream_t s) {
  const bool is3d = r.nz > 1;
  IcOut o{{f[0], f[1], f[2], f[3]}, {0.0, 0.0}};
  if (r.profile == 1)
    for (int k = 0; k < 2; k++)
      o.bellA[k] = ic_bell_amplitude(r.bell_sigma[k], r.bell_range[0], r.bell_range[1],
                                     r.matrix[k], r.enrich[k]);
  dim3 grid((r.nx + 31) / 32, (r.ny + 7) / 8, is3d ? r.nz : 1);
  k_ic_fill<<<grid, 256, 0, s>>>(r, o, is3d ? 1 : 0);
  return cudaGetLastError();
}

}  // namespace pfa

extern "C" {

int pfa_ic_generate(const pfa_ic_recipe* r, double* conc_Cr, double* conc_Nb, double* phi_del,
                    double* phi_lav, void* stream) {
  const char* msg = pfa::ic_check(r);
  if (!msg && (!conc_Cr || !conc_Nb || !phi_del || !phi_lav))
    msg = "pfa_ic_generate: null field";
  if (msg) {
    std::fprintf(stderr, "pfa_gb300: %s\n", msg);
    pfa::set_error(PFA_EINVAL, msg);
    return PFA_EINVAL;
  }
  double* const f[4] = {conc_Cr, conc_Nb, phi_del, phi_lav};
  const cudaError_t e = pfa::launch_ic_fill(*r, f, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    char buf[256];
    std::snprintf(buf, sizeof(buf), "pfa_ic_generate: %s", cudaGetErrorString(e));
    std::fprintf(stderr, "CUDA Runtime Error: %s\n", buf);
    pfa::set_error(PFA_ECUDA, buf);
    return PFA_ECUDA;
  }
  return 0;
}

}  // extern "C"
