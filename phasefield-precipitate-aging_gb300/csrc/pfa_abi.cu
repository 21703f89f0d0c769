// pfa_abi.cu -- the reference's GPU entry points and their extern "C" mirror.
//
// Implements the host functions of src/data.cuh and src/discretization.cuh
// (usnistgov/phasefield-precipitate-aging) with the same signatures and
// CudaData layout, on top of the fused kernels of this library.  State the
// reference's structure has no room for (precision, FP32 buffers, scratch
// buffers, captured graphs, nucleation counters) lives in a table keyed by
// the caller's CudaData pointer.
//
// Threading: one host thread per CudaData, as in the reference; the table
// itself is guarded by a mutex.  All work of one CudaData is ordered on its
// stream str_A.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "pfa_gb300.h"
#include "pfa_reference_abi.h"

#include "pfa_internal.h"
#include "pfa_kernels.h"
#include "pfa_model.h"
#include "pfa_nucleation.h"
#include "pfa_reduce.h"

namespace pfa {

// ---------------------------------------------------------------------------
// errors
static int g_err = 0;
static char g_msg[512] = "";

void set_error(int code, const char* where) {
  g_err = code;
  std::snprintf(g_msg, sizeof(g_msg), "%s", where ? where : "");
}

static int cuda_fail(cudaError_t e, const char* what) {
  std::fprintf(stderr, "CUDA Runtime Error: %s (%s)\n", cudaGetErrorString(e), what);
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  set_error(PFA_ECUDA, buf);
  return PFA_ECUDA;
}

static int fail(int code, const char* what) {
  std::fprintf(stderr, "pfa_gb300: %s\n", what);
  set_error(code, what);
  return code;
}

#define CK(expr)                                           \
  do {                                                     \
    cudaError_t e_ = (expr);                               \
    if (e_ != cudaSuccess) return cuda_fail(e_, #expr);    \
  } while (0)

// ---------------------------------------------------------------------------
struct GraphEntry {
  int precision, len, nuc_first, cur;
  const void* ptrs[8];
  double dt, alpha;
  cudaGraphExec_t exec;
};

struct State {
  int nx = 0, ny = 0, Nx = 0, Ny = 0;
  int mode = PFA_MODE_FUSED, precision = PFA_FP64;
  double mask9[9] = {};
  bool five_point = true;
  bool symmetric = true;  // corners, left / right and upper / lower weights equal (FP32 form)
  bool zero_sum = true;   // the nine weights sum to zero (up to rounding)
  ModelConst m{};
  FastCoef fk{};
  cudaStream_t st = nullptr;
  // FP32 precision form: two buffer sets (fields + compensation)
  int pitch32 = 0;      // records per row
  float* f32mem = nullptr;
  float* recA[2] = {};  // {x_Cr, x_Nb, phi_del, phi_lav} records, ping-pong
  float* recB[2] = {};  // Kahan compensation records (packed counts or FP32)
  int cur = 0;
  bool f32_live = false;
  // nucleation
  uint64_t seed = 42;
  uint64_t calls = 0;
  int geometry = PFA_NUC_REFERENCE_GEOMETRY;
  int nuc_interval = 0;
  double nuc_sigma[2] = {0.13, 0.13}, nuc_unit_a = 0.352e-9, nuc_d[3] = {0, 0, 0}, nuc_dt = 0;
  uint64_t step_counter = 0;
  // scratch (event buffer, counters, partial sums)
  NucEvent* ev = nullptr;
  unsigned* ev_count = nullptr;  // [0] events, [1] listed cells
  int* ev_status = nullptr;
  unsigned long long* call_dev = nullptr;
  long long* cand = nullptr;  // cells left to the FP64 nucleation decision
  int cand_cap = 0;
  double* sum_partial = nullptr;
  double* sum_out = nullptr;
  cudaEvent_t xev[8] = {};  // chunked transfers (created on first use)
  cudaEvent_t xdone = nullptr;  // the read-out's last copy on str_B
  double* nrg_map[2] = {};  // per-node chemical / gradient energy (on request)
  // variable-mobility Cahn-Hilliard (pfa_set_mobility): the compat stages'
  // 16 coefficient arrays (allocated on first use) and the spacing of the
  // divergence (the last device_laplacian call's, else from the mask)
  int varmob = 0;
  double* mob[16] = {};
  double dxy[2] = {0.0, 0.0};
  std::vector<GraphEntry> graphs;
};

static std::mutex g_mu;
static std::unordered_map<const CudaData*, State*> g_tab;

static State* lookup(const CudaData* dev) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_tab.find(dev);
  return it == g_tab.end() ? nullptr : it->second;
}

static void drop_graphs(State* s) {
  for (auto& g : s->graphs) cudaGraphExecDestroy(g.exec);
  s->graphs.clear();
}

// ---------------------------------------------------------------------------
static int init_core(CudaData* dev, int nx, int ny, int nm, const double* mask,
                     const double* kappa, const double* omega, const double* Lmob,
                     const double* D_Cr, const double* D_Nb, const double* cr, const double* nb,
                     const double* pd, const double* pl);
static int free_core(CudaData* dev);

static int alloc_field(double** p, size_t n) {
  CK(cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(double)));
  return 0;
}

static int ensure_fict(CudaData* dev, State* s) {
  const size_t n = size_t(s->nx) * s->ny;
  double** arrs[6] = {&dev->conc_Cr_gam, &dev->conc_Nb_gam, &dev->conc_Cr_del,
                      &dev->conc_Nb_del, &dev->conc_Cr_lav, &dev->conc_Nb_lav};
  for (auto a : arrs)
    if (!*a && alloc_field(a, n)) return PFA_ECUDA;
  return 0;
}

// FP32 form buffers: two record sets (A 16 bytes, B 16 bytes per cell so
// either precision variant fits), Ny rows of pitch32 records (a multiple of
// 32), interior only; every array starts on a 256-byte boundary.
static int ensure_f32(State* s) {
  if (s->f32mem) return 0;
  s->pitch32 = ((s->Nx + 31) / 32) * 32;
  const size_t per = ((size_t(s->pitch32) * s->Ny * 4 + 63) / 64) * 64;  // floats per array
  CK(cudaMalloc(reinterpret_cast<void**>(&s->f32mem), per * 4 * sizeof(float)));
  CK(cudaMemsetAsync(s->f32mem, 0, per * 4 * sizeof(float), s->st));
  for (int b = 0; b < 2; b++) {
    s->recA[b] = s->f32mem + per * (2 * b);
    s->recB[b] = s->f32mem + per * (2 * b + 1);
  }
  return 0;
}

static ConvArgs conv_args(CudaData* dev, State* s) {
  ConvArgs c{};
  c.f64[0] = dev->conc_Cr_old;
  c.f64[1] = dev->conc_Nb_old;
  c.f64[2] = dev->phi_del_old;
  c.f64[3] = dev->phi_lav_old;
  const bool kphi = s->precision == PFA_FP32_KPHI;
  c.A = s->recA[s->cur];
  c.B = s->recB[s->cur];
  c.pack = !kphi;
  c.Nx = s->Nx;
  c.Ny = s->Ny;
  c.pitch64 = s->nx;
  c.pitch32 = s->pitch32;
  return c;
}

// FP64 *_old -> FP32 state (when the FP32 state is not authoritative yet)
static int f32_import(CudaData* dev, State* s) {
  if (s->f32_live) return 0;
  if (int r = ensure_f32(s)) return r;
  s->cur = 0;
  CK(launch_import_f32(conv_args(dev, s), s->st));
  s->f32_live = true;
  return 0;
}

// FP32 state -> FP64 *_old (ghost ring mirrored)
static int f32_export(CudaData* dev, State* s) {
  if (!s->f32_live) return 0;
  CK(launch_export_f32(conv_args(dev, s), s->st));
  return 0;
}

static Step2DArgs step_args(State* s, double alpha, double dt) {
  Step2DArgs a{};
  a.Nx = s->Nx;
  a.Ny = s->Ny;
  a.m = s->m;
  a.m.alpha = alpha;
  a.m.dt = dt;
  std::memcpy(a.mask9, s->mask9, sizeof(a.mask9));
  a.nine = !s->five_point;
  a.varmob = s->varmob;
  a.k = s->fk;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) a.dtD[i][j] = float(dt * s->m.D[i][j]);
  for (int i = 0; i < 2; i++) {
    a.dtL[i] = float(dt * s->m.L[i]);
    a.om2[i] = float(2.0 * s->m.omega[i]);
    a.kap[i] = float(s->m.kappa[i]);
  }
  a.alpha2 = float(2.0 * alpha);
  a.idx2f[0] = float(s->m.idx2[0]);
  a.idx2f[1] = float(s->m.idx2[1]);
  // the FP32 form's general (9-point) Laplacian weights
  double sum = 0.0;
  for (double w : s->mask9) sum += w;
  a.lap9[0] = float(s->mask9[3]);
  a.lap9[1] = float(s->mask9[1]);
  a.lap9[2] = float(s->mask9[0]);
  a.lap9[3] = float(sum);
  for (int k = 0; k < 2; k++) a.lap9xe[k] = float(sum * kXe[0][k]);
  // the FP32 form's variable-mobility step takes the diffusivity matrix
  // already scaled by dt / (2 dx^2) (the x faces' weight of the divergence)
  const double r2x = 0.5 * dt * s->m.idx2[0];
  a.vm_pre[0] = float(kMobPreNb * r2x);
  a.vm_pre[1] = float(kMobPreCr * r2x);
  a.vm_pre[2] = float(kMobPreNi * r2x);
  a.vm_qy = s->m.idx2[0] > 0.0 ? float(s->m.idx2[1] / s->m.idx2[0]) : 0.0f;
  return a;
}

// One fused step: FP64 old -> new, or FP32 cur -> 1 - cur.
static int fused_step(CudaData* dev, State* s, double alpha, double dt) {
  Step2DArgs a = step_args(s, alpha, dt);
  if (s->precision == PFA_FP64) {
    a.in[0] = dev->conc_Cr_old;
    a.in[1] = dev->conc_Nb_old;
    a.in[2] = dev->phi_del_old;
    a.in[3] = dev->phi_lav_old;
    a.out[0] = dev->conc_Cr_new;
    a.out[1] = dev->conc_Nb_new;
    a.out[2] = dev->phi_del_new;
    a.out[3] = dev->phi_lav_new;
    a.pitch = s->nx;
    a.write_halo = 1;
    CK(launch_step2d_f64(a, s->st));
    return 0;
  }
  if (!s->symmetric)
    return fail(PFA_EINVAL, "the FP32 form needs a symmetric mask (equal corners, left / right, upper / lower)");
  if (int r = f32_import(dev, s)) return r;
  const int c = s->cur, n = 1 - c;
  a.in[0] = s->recA[c];
  a.in[1] = s->recB[c];
  a.out[0] = s->recA[n];
  a.out[1] = s->recB[n];
  a.pitch = s->pitch32;
  a.full_comp = s->precision == PFA_FP32_KPHI;
  // the 5-point FP32 kernel takes the centre weight as -2 (left + upper);
  // a mask whose weights do not sum to zero goes through the general form
  a.nine = !s->five_point || !s->zero_sum;
  CK(launch_step2d_f32(a, s->st));
  s->cur = n;
  return 0;
}

// Nucleation on the state after a step: FP64 *_new (before the caller's swap)
// or the current FP32 buffers.
static int nucleate(CudaData* dev, State* s, double sig_d, double sig_l, double unit_a, double dx,
                    double dy, double dz, double dt) {
  NucArgs a{};
  if (s->precision == PFA_FP64) {
    a.f[0] = dev->conc_Cr_new;
    a.f[1] = dev->conc_Nb_new;
    a.f[2] = dev->phi_del_new;
    a.f[3] = dev->phi_lav_new;
    a.pitch = s->nx;
    a.is_f32 = 0;
    a.stride = 1;
  } else {
    if (int r = f32_import(dev, s)) return r;
    for (int k = 0; k < 4; k++) a.f[k] = s->recA[s->cur] + k;
    a.comp = s->recB[s->cur];
    a.pack = s->precision == PFA_FP32;
    a.stride = 4;
    a.pitch = s->pitch32;
    a.is_f32 = 1;
    a.compact = 1;
  }
  a.Nx = s->Nx;
  a.Ny = s->Ny;
  a.sigma[0] = sig_d;
  a.sigma[1] = sig_l;
  // src/discretization.cu:1206: the reference wrapper hands the kernel
  // dx * nx and dy * ny; the fixed geometry passes the spacing itself.
  const double kdx = s->geometry == PFA_NUC_REFERENCE_GEOMETRY ? dx * s->nx : dx;
  const double kdy = s->geometry == PFA_NUC_REFERENCE_GEOMETRY ? dy * s->ny : dy;
  if (const char* msg = nucleation_constants(a, kdx, kdy, dz, dt, unit_a))
    return fail(PFA_EINVAL, msg);
  a.seed = s->seed;
  a.call_ptr = s->call_dev;
  a.events = s->ev;
  a.keys = reinterpret_cast<unsigned long long*>(s->ev + kNucCap);
  a.count = s->ev_count;
  a.status = s->ev_status;
  a.cap = kNucCap;
  a.cand = s->cand;
  a.cand_cap = s->cand_cap;
  CK(launch_nucleation(a, s->st));
  s->calls++;
  return 0;
}

static int run_step_compat(CudaData* dev, State* s, double alpha, double dt);

static int swap_ptrs(CudaData* dev) {
  std::swap(dev->conc_Cr_old, dev->conc_Cr_new);
  std::swap(dev->conc_Nb_old, dev->conc_Nb_new);
  std::swap(dev->phi_del_old, dev->phi_del_new);
  std::swap(dev->phi_lav_old, dev->phi_lav_new);
  return 0;
}

// `len` steps; nucleation after the first one when nuc_first.  Leaves the
// latest fields in *_old (FP64) or f32[cur] (FP32), as the caller-side
// swaps of src/main.cpp:318-321 would.
static int launch_chunk(CudaData* dev, State* s, int len, bool nuc_first, double alpha, double dt) {
  for (int k = 0; k < len; k++) {
    if (int r = fused_step(dev, s, alpha, dt)) return r;
    if (k == 0 && nuc_first)
      if (int r = nucleate(dev, s, s->nuc_sigma[0], s->nuc_sigma[1], s->nuc_unit_a, s->nuc_d[0],
                           s->nuc_d[1], s->nuc_d[2], s->nuc_dt))
        return r;
    if (s->precision == PFA_FP64) swap_ptrs(dev);
  }
  return 0;
}

static int run_chunk(CudaData* dev, State* s, int len, bool nuc_first, double alpha, double dt) {
  if (len % 2 != 0 || len < 2) return launch_chunk(dev, s, len, nuc_first, alpha, dt);
  if (s->precision != PFA_FP64 && !s->f32_live)
    if (int r = f32_import(dev, s)) return r;
  GraphEntry key{};
  key.precision = s->precision;
  key.len = len;
  key.nuc_first = nuc_first;
  key.cur = s->cur;
  const void* p[8] = {dev->conc_Cr_old, dev->conc_Cr_new, dev->conc_Nb_old, dev->conc_Nb_new,
                      dev->phi_del_old, dev->phi_del_new, dev->phi_lav_old, dev->phi_lav_new};
  std::memcpy(key.ptrs, p, sizeof(p));
  key.dt = dt;
  key.alpha = alpha;
  cudaGraphExec_t exec = nullptr;
  for (auto& g : s->graphs)
    if (g.precision == key.precision && g.len == len && g.nuc_first == key.nuc_first &&
        g.cur == key.cur && !std::memcmp(g.ptrs, key.ptrs, sizeof(p)) && g.dt == dt &&
        g.alpha == alpha)
      exec = g.exec;
  const int cur0 = s->cur;
  const uint64_t calls0 = s->calls;
  if (!exec) {
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    const int r = launch_chunk(dev, s, len, nuc_first, alpha, dt);
    const cudaError_t e = cudaStreamEndCapture(s->st, &graph);
    // capture only recorded the launches: restore the host-side bookkeeping
    // (the ping-pong pointers and counters launch_chunk advanced), on every
    // exit, so the handle still names the live fields when capture failed
    double** slots[8] = {&dev->conc_Cr_old, &dev->conc_Cr_new, &dev->conc_Nb_old,
                         &dev->conc_Nb_new, &dev->phi_del_old, &dev->phi_del_new,
                         &dev->phi_lav_old, &dev->phi_lav_new};
    for (int k = 0; k < 8; k++) *slots[k] = const_cast<double*>(static_cast<const double*>(p[k]));
    s->cur = cur0;
    s->calls = calls0;
    if (r || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return r ? r : cuda_fail(e, "cudaStreamEndCapture");
    }
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) return cuda_fail(ei, "cudaGraphInstantiate");
    key.exec = exec;
    if (s->graphs.size() >= 8) drop_graphs(s);
    s->graphs.push_back(key);
  }
  CK(cudaGraphLaunch(exec, s->st));
  // an even number of steps returns every ping-pong pointer to its place
  if (nuc_first) s->calls++;
  return 0;
}

static int run_core(CudaData* dev, State* s, int nsteps, double alpha, double dt) {
  if (nsteps < 0) return fail(PFA_EINVAL, "negative step count");
  if (s->mode == PFA_MODE_COMPAT) {
    for (int k = 0; k < nsteps; k++) {
      if (int r = run_step_compat(dev, s, alpha, dt)) return r;
      if (s->nuc_interval > 0 && s->step_counter % s->nuc_interval == 0)
        if (int r = nucleate(dev, s, s->nuc_sigma[0], s->nuc_sigma[1], s->nuc_unit_a, s->nuc_d[0],
                             s->nuc_d[1], s->nuc_d[2], s->nuc_dt))
          return r;
      swap_ptrs(dev);
      s->step_counter++;
    }
    return 0;
  }
  int remaining = nsteps;
  while (remaining > 0) {
    int len;
    bool nuc_first = false;
    if (s->nuc_interval > 0) {
      const int phase = int(s->step_counter % uint64_t(s->nuc_interval));
      nuc_first = phase == 0;
      len = std::min(remaining, s->nuc_interval - phase);
    } else {
      len = std::min(remaining, 100);
    }
    if (len > 1 && len % 2) {
      // peel one step so the graph sees an even count
      if (int r = launch_chunk(dev, s, 1, nuc_first, alpha, dt)) return r;
      s->step_counter += 1;
      remaining -= 1;
      len -= 1;
      nuc_first = false;
    }
    if (int r = run_chunk(dev, s, len, nuc_first, alpha, dt)) return r;
    s->step_counter += uint64_t(len);
    remaining -= len;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// compat-mode stages
static StageArgs stage_args(CudaData* dev, State* s) {
  StageArgs a{};
  a.f[0] = dev->conc_Cr_old;
  a.f[1] = dev->conc_Nb_old;
  a.f[2] = dev->phi_del_old;
  a.f[3] = dev->phi_lav_old;
  a.o[0] = dev->conc_Cr_new;
  a.o[1] = dev->conc_Nb_new;
  a.o[2] = dev->phi_del_new;
  a.o[3] = dev->phi_lav_new;
  a.gam[0] = dev->conc_Cr_gam;
  a.gam[1] = dev->conc_Nb_gam;
  a.del[0] = dev->conc_Cr_del;
  a.del[1] = dev->conc_Nb_del;
  a.lav[0] = dev->conc_Cr_lav;
  a.lav[1] = dev->conc_Nb_lav;
  a.nx = s->nx;
  a.ny = s->ny;
  a.m = s->m;
  std::memcpy(a.mask9, s->mask9, sizeof(a.mask9));
  for (int k = 0; k < 16; k++) a.mob[k] = s->mob[k];
  a.dxy[0] = s->dxy[0];
  a.dxy[1] = s->dxy[1];
  a.varmob = s->varmob;
  return a;
}

static int st_boundaries(CudaData* dev, State* s) {
  double* f[4] = {dev->conc_Cr_old, dev->conc_Nb_old, dev->phi_del_old, dev->phi_lav_old};
  for (double* p : f) CK(launch_bc(p, s->nx, s->ny, s->st));
  double* g[6] = {dev->conc_Cr_gam, dev->conc_Nb_gam, dev->conc_Cr_del,
                  dev->conc_Nb_del, dev->conc_Cr_lav, dev->conc_Nb_lav};
  for (double* p : g)
    if (p) CK(launch_bc(p, s->nx, s->ny, s->st));
  return 0;
}

static int st_fictitious(CudaData* dev, State* s) {
  if (int r = ensure_fict(dev, s)) return r;
  CK(launch_fictitious(stage_args(dev, s), s->st));
  return 0;
}

static int st_fict_boundaries(CudaData* dev, State* s) {
  if (int r = ensure_fict(dev, s)) return r;
  double* g[6] = {dev->conc_Cr_gam, dev->conc_Nb_gam, dev->conc_Cr_del,
                  dev->conc_Nb_del, dev->conc_Cr_lav, dev->conc_Nb_lav};
  for (double* p : g) CK(launch_bc(p, s->nx, s->ny, s->st));
  return 0;
}

// the variable-mobility coefficients at every cell from the old fields and
// the fictitious compositions (device_mobilities, src/discretization.cu:297-358)
static int st_mobilities(CudaData* dev, State* s) {
  if (int r = ensure_fict(dev, s)) return r;
  const size_t n = size_t(s->nx) * s->ny;
  for (auto& p : s->mob)
    if (!p && alloc_field(&p, n)) return PFA_ECUDA;
  CK(launch_mobility(stage_args(dev, s), s->st));
  return 0;
}

// mobility_boundaries (declared, never defined by the reference): the
// zero-flux fill of the coefficients' ghost ring
static int st_mob_boundaries(CudaData* dev, State* s) {
  (void)dev;
  for (double* p : s->mob)
    if (p) CK(launch_bc(p, s->nx, s->ny, s->st));
  return 0;
}

// device_laplacian (src/discretization.cu:780-841): the mask convolution of
// the phases and of the gamma compositions, or, with the variable mobility,
// of the phases and chemical_convolution_Cr/Nb (the reference's commented
// launches) for the compositions -- with the coefficients computed here, so
// that a loop that never calls device_mobilities still gets them
static int st_laplacian(CudaData* dev, State* s) {
  if (int r = ensure_fict(dev, s)) return r;
  CK(launch_convolution(dev->phi_del_old, dev->phi_del_new, s->nx, s->ny, s->mask9, s->st));
  CK(launch_convolution(dev->phi_lav_old, dev->phi_lav_new, s->nx, s->ny, s->mask9, s->st));
  if (s->varmob) {
    if (int r = st_mobilities(dev, s)) return r;
    if (int r = st_mob_boundaries(dev, s)) return r;
    CK(launch_chem_convolution(stage_args(dev, s), s->st));
    return 0;
  }
  CK(launch_convolution(dev->conc_Cr_gam, dev->conc_Cr_new, s->nx, s->ny, s->mask9, s->st));
  CK(launch_convolution(dev->conc_Nb_gam, dev->conc_Nb_new, s->nx, s->ny, s->mask9, s->st));
  return 0;
}

static int st_lap_boundaries(CudaData* dev, State* s) {
  double* f[4] = {dev->conc_Cr_new, dev->conc_Nb_new, dev->phi_del_new, dev->phi_lav_new};
  for (double* p : f) CK(launch_bc(p, s->nx, s->ny, s->st));
  return 0;
}

static int st_evolution(CudaData* dev, State* s, double alpha, double dt) {
  StageArgs a = stage_args(dev, s);
  a.m.alpha = alpha;
  a.m.dt = dt;
  CK(launch_evolution(a, s->st));
  return 0;
}

static int run_step_compat(CudaData* dev, State* s, double alpha, double dt) {
  if (s->precision != PFA_FP64) return fail(PFA_EINVAL, "compat mode is FP64 only");
  if (int r = st_boundaries(dev, s)) return r;
  if (int r = st_fictitious(dev, s)) return r;
  if (int r = st_fict_boundaries(dev, s)) return r;
  if (int r = st_laplacian(dev, s)) return r;
  if (int r = st_lap_boundaries(dev, s)) return r;
  return st_evolution(dev, s, alpha, dt);
}

// ---------------------------------------------------------------------------
static int init_core(CudaData* dev, int nx, int ny, int nm, const double* mask,
                     const double* kappa, const double* omega, const double* Lmob,
                     const double* D_Cr, const double* D_Nb, const double* cr, const double* nb,
                     const double* pd, const double* pl) {
  if (!dev || !mask || !kappa || !omega || !Lmob || !D_Cr || !D_Nb)
    return fail(PFA_EINVAL, "init_cuda: null argument");
  if (nm != 3) return fail(PFA_EINVAL, "init_cuda: nm must be 3");
  if (nx < 3 || ny < 3) return fail(PFA_EINVAL, "init_cuda: grid smaller than 3 x 3");
  if (lookup(dev)) free_core(dev);
  std::memset(dev, 0, sizeof(*dev));
  State* s = new State();
  s->nx = nx;
  s->ny = ny;
  s->Nx = nx - 2;
  s->Ny = ny - 2;
  std::memcpy(s->mask9, mask, sizeof(s->mask9));
  s->five_point = mask[0] == 0.0 && mask[2] == 0.0 && mask[6] == 0.0 && mask[8] == 0.0;
  s->symmetric = mask[0] == mask[2] && mask[0] == mask[6] && mask[0] == mask[8] &&
                 mask[1] == mask[7] && mask[3] == mask[5];
  {
    double sum = 0.0;
    for (int k = 0; k < 9; k++) sum += mask[k];
    s->zero_sum = std::fabs(sum) <= 1e-12 * std::fabs(mask[4]);
  }
  for (int i = 0; i < 2; i++) {
    s->m.D[0][i] = D_Cr[i];
    s->m.D[1][i] = D_Nb[i];
    s->m.kappa[i] = kappa[i];
    s->m.omega[i] = omega[i];
    s->m.L[i] = Lmob[i];
  }
  s->m.mask[0] = mask[1];
  s->m.mask[1] = mask[3];
  s->m.mask[2] = mask[4];
  s->m.mask[3] = mask[5];
  s->m.mask[4] = mask[7];
  s->m.idx2[0] = mask[3];  // left: 1/dx^2 (src/mesh.cpp:191)
  s->m.idx2[1] = mask[1];  // upper: 1/dy^2 (src/mesh.cpp:190)
  s->dxy[0] = mask[3] > 0.0 ? 1.0 / std::sqrt(mask[3]) : 0.0;
  s->dxy[1] = mask[1] > 0.0 ? 1.0 / std::sqrt(mask[1]) : 0.0;
  s->m.idx2[2] = 0.0;
  model_fast_coef(&s->fk);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_tab[dev] = s;
  }
  CK(cudaStreamCreateWithFlags(&dev->str_A, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&dev->str_B, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&dev->str_C, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&dev->str_D, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&dev->ev_A, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&dev->ev_B, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&dev->ev_C, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&dev->ev_D, cudaEventDisableTiming));
  s->st = dev->str_A;
  const size_t n = size_t(nx) * ny;
  double** main_f[8] = {&dev->conc_Cr_old, &dev->conc_Cr_new, &dev->conc_Nb_old,
                        &dev->conc_Nb_new, &dev->phi_del_old, &dev->phi_del_new,
                        &dev->phi_lav_old, &dev->phi_lav_new};
  for (auto p : main_f)
    if (alloc_field(p, n)) return PFA_ECUDA;
  CK(cudaMalloc(reinterpret_cast<void**>(&s->ev), nucleation_event_bytes()));
  CK(cudaMalloc(reinterpret_cast<void**>(&s->ev_count), 2 * sizeof(unsigned)));
  s->cand_cap = nucleation_cand_cap(n);
  CK(cudaMalloc(reinterpret_cast<void**>(&s->cand), sizeof(long long) * size_t(s->cand_cap)));
  CK(cudaMalloc(reinterpret_cast<void**>(&s->ev_status), sizeof(int)));
  CK(cudaMalloc(reinterpret_cast<void**>(&s->call_dev), sizeof(unsigned long long)));
  CK(cudaMalloc(reinterpret_cast<void**>(&s->sum_partial), sizeof(double) * kSumBlocks * 5));
  CK(cudaMalloc(reinterpret_cast<void**>(&s->sum_out), sizeof(double) * 5));
  CK(cudaMemsetAsync(s->ev_count, 0, 2 * sizeof(unsigned), s->st));
  CK(cudaMemsetAsync(s->ev_status, 0, sizeof(int), s->st));
  CK(cudaMemsetAsync(s->call_dev, 0, sizeof(unsigned long long), s->st));
  static bool nuc_ready = false;
  if (!nuc_ready) {
    CK(nucleation_setup());
    CK(prepare_step2d_f32());
    CK(prepare_step2d_f64());
    nuc_ready = true;
  }
  if (cr) {
    const double* src[4] = {cr, nb, pd, pl};
    double* dst[4] = {dev->conc_Cr_old, dev->conc_Nb_old, dev->phi_del_old, dev->phi_lav_old};
    for (int k = 0; k < 4; k++)
      CK(cudaMemcpyAsync(dst[k], src[k], n * sizeof(double), cudaMemcpyHostToDevice, s->st));
  }
  CK(cudaStreamSynchronize(s->st));
  return 0;
}

static int free_core(CudaData* dev) {
  State* s;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_tab.find(dev);
    if (it == g_tab.end()) return fail(PFA_ESTATE, "free_cuda: unknown CudaData");
    s = it->second;
    g_tab.erase(it);
  }
  if (s->st) cudaStreamSynchronize(s->st);
  if (dev->str_B) cudaStreamSynchronize(dev->str_B);  // an asynchronous read-out
  drop_graphs(s);
  double* f[16] = {dev->conc_Cr_old, dev->conc_Cr_new, dev->conc_Nb_old, dev->conc_Nb_new,
                   dev->phi_del_old, dev->phi_del_new, dev->phi_lav_old, dev->phi_lav_new,
                   dev->conc_Cr_gam, dev->conc_Nb_gam, dev->conc_Cr_del, dev->conc_Nb_del,
                   dev->conc_Cr_lav, dev->conc_Nb_lav, dev->conc_Ni, dev->phi};
  int rc = 0;
  for (double* p : f)
    if (p && cudaFree(p) != cudaSuccess) rc = PFA_ECUDA;
  cudaFree(s->f32mem);
  cudaFree(s->ev);
  cudaFree(s->ev_count);
  cudaFree(s->cand);
  cudaFree(s->ev_status);
  cudaFree(s->call_dev);
  cudaFree(s->sum_partial);
  cudaFree(s->sum_out);
  cudaFree(s->nrg_map[0]);
  cudaFree(s->nrg_map[1]);
  for (double* p : s->mob) cudaFree(p);
  for (cudaEvent_t e : s->xev)
    if (e) cudaEventDestroy(e);
  if (s->xdone) cudaEventDestroy(s->xdone);
  cudaStream_t st[4] = {dev->str_A, dev->str_B, dev->str_C, dev->str_D};
  for (auto x : st)
    if (x) cudaStreamDestroy(x);
  cudaEvent_t ev[4] = {dev->ev_A, dev->ev_B, dev->ev_C, dev->ev_D};
  for (auto x : ev)
    if (x) cudaEventDestroy(x);
  std::memset(dev, 0, sizeof(*dev));
  delete s;
  if (rc) return fail(rc, "free_cuda: cudaFree failed");
  return 0;
}

// Read-outs of the FP32 form move the FP64 fields in row bands so that the
// layout conversion of one band overlaps the copy of the one before: the
// conversions run on the library stream, the copies on the CudaData's second
// stream (str_B), ordered band by band with events.
constexpr int kXferBands = 8;

static int ensure_xfer(State* s) {
  if (s->xev[0]) return 0;
  for (int i = 0; i < kXferBands; i++)
    CK(cudaEventCreateWithFlags(&s->xev[i], cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&s->xdone, cudaEventDisableTiming));
  return 0;
}

// interior rows whose FP64 row (ghost-ring layout) lies in [r0, r1)
static void band_rows(const State* s, int r0, int r1, ConvArgs& c) {
  c.y0 = r0 > 0 ? r0 - 1 : 0;
  c.y1 = r1 - 1 < s->Ny ? r1 - 1 : s->Ny;
}

// wait = false: enqueue only; later work on the library stream (uploads,
// steps, exports that overwrite the FP64 fields) is ordered after the copies
static int read_core(CudaData* dev, double* cr, double* nb, double* pd, double* pl, int nx,
                     int ny, bool wait) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "read_out_result: unknown CudaData");
  if (nx != s->nx || ny != s->ny) return fail(PFA_EINVAL, "read_out_result: size mismatch");
  double* dst[4] = {cr, nb, pd, pl};
  const double* src[4] = {dev->conc_Cr_old, dev->conc_Nb_old, dev->phi_del_old, dev->phi_lav_old};
  if (s->precision != PFA_FP64 && s->f32_live && dev->str_B) {
    if (int r = ensure_xfer(s)) return r;
    // at least two rows per band: the first band then holds the bottom ghost
    // row together with the interior row that writes it
    const int rows = std::max(2, (ny + kXferBands - 1) / kXferBands);
    for (int i = 0; i < kXferBands; i++) {
      const int r0 = i * rows, r1 = r0 + rows < ny ? r0 + rows : ny;
      if (r0 >= r1) break;
      ConvArgs c = conv_args(dev, s);
      band_rows(s, r0, r1, c);
      // a band's rows are written by its own interior rows (ghost rows by the
      // first and last interior row, which lie in the first and last band)
      if (c.y1 > c.y0) CK(launch_export_f32(c, s->st));
      CK(cudaEventRecord(s->xev[i], s->st));
      CK(cudaStreamWaitEvent(dev->str_B, s->xev[i], 0));
      const size_t off = size_t(r0) * nx, bytes = size_t(r1 - r0) * nx * sizeof(double);
      for (int k = 0; k < 4; k++)
        if (dst[k])
          CK(cudaMemcpyAsync(dst[k] + off, src[k] + off, bytes, cudaMemcpyDeviceToHost, dev->str_B));
    }
    CK(cudaEventRecord(s->xdone, dev->str_B));
    CK(cudaStreamWaitEvent(s->st, s->xdone, 0));
    if (wait) CK(cudaStreamSynchronize(dev->str_B));
    return 0;
  }
  if (int r = f32_export(dev, s)) return r;
  const size_t n = size_t(nx) * ny;
  for (int k = 0; k < 4; k++)
    if (dst[k]) CK(cudaMemcpyAsync(dst[k], src[k], n * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  if (wait) CK(cudaStreamSynchronize(s->st));
  return 0;
}

// wait = false: enqueue only (the sources are read asynchronously)
static int upload_core(CudaData* dev, const double* cr, const double* nb, const double* pd,
                       const double* pl, int nx, int ny, bool wait) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "upload: unknown CudaData");
  if (nx != s->nx || ny != s->ny) return fail(PFA_EINVAL, "upload: size mismatch");
  const size_t n = size_t(nx) * ny;
  const double* src[4] = {cr, nb, pd, pl};
  double* dst[4] = {dev->conc_Cr_old, dev->conc_Nb_old, dev->phi_del_old, dev->phi_lav_old};
  for (int k = 0; k < 4; k++)
    CK(cudaMemcpyAsync(dst[k], src[k], n * sizeof(double), cudaMemcpyHostToDevice, s->st));
  if (s->precision != PFA_FP64) {
    // convert now (whole-field copies: each extra copy call costs ~15 us, more
    // than banding the conversion behind the copies would save)
    if (int r = ensure_f32(s)) return r;
    s->cur = 0;
    CK(launch_import_f32(conv_args(dev, s), s->st));
    if (wait) CK(cudaStreamSynchronize(s->st));  // page-locked sources are read asynchronously
    s->f32_live = true;
    return 0;
  }
  if (wait) CK(cudaStreamSynchronize(s->st));  // page-locked sources are read asynchronously
  s->f32_live = false;
  return 0;
}

static int dataviz_core(CudaData* dev, double* cr, double* nb, double* ni, double* pd, double* pl,
                        double* phi) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "device_dataviz: unknown CudaData");
  const size_t n = size_t(s->nx) * s->ny;
  if (!dev->conc_Ni && alloc_field(&dev->conc_Ni, n)) return PFA_ECUDA;
  if (!dev->phi && alloc_field(&dev->phi, n)) return PFA_ECUDA;
  if (int r = f32_export(dev, s)) return r;
  CK(launch_dataviz(dev->conc_Cr_old, dev->conc_Nb_old, dev->phi_del_old, dev->phi_lav_old,
                    dev->conc_Ni, dev->phi, s->nx, s->ny, s->st));
  double* dst[6] = {cr, nb, ni, pd, pl, phi};
  const double* src[6] = {dev->conc_Cr_old, dev->conc_Nb_old, dev->conc_Ni,
                          dev->phi_del_old, dev->phi_lav_old, dev->phi};
  for (int k = 0; k < 6; k++)
    if (dst[k]) CK(cudaMemcpyAsync(dst[k], src[k], n * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return 0;
}

// nucleation status word: read (and clear) after the stream drains
static int check_nucleation_status(State* s) {
  int st = 0;
  CK(cudaMemcpyAsync(&st, s->ev_status, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (st) {
    CK(cudaMemsetAsync(s->ev_status, 0, sizeof(int), s->st));
    if (st == 2) return fail(PFA_EINVAL, "nucleation: a nucleus radius exceeded 256 cells (not painted)");
    return fail(PFA_EOVERFLOW, "nucleation: more events than the event buffer holds");
  }
  return 0;
}

}  // namespace pfa

using namespace pfa;

// ===========================================================================
// The reference's C++ entry points (src/data.cuh, src/discretization.cuh)
cudaError_t checkCuda(cudaError_t result) {
  if (result != cudaSuccess) {
    std::fprintf(stderr, "CUDA Runtime Error: %s\n", cudaGetErrorString(result));
    set_error(PFA_ECUDA, cudaGetErrorString(result));
  }
  return result;
}

void init_cuda(struct HostData* host, const int nx, const int ny, const int nm, const fp_t* kappa,
               const fp_t* omega, const fp_t* Lmob, const fp_t* D_Cr, const fp_t* D_Nb,
               struct CudaData* dev) {
  if (!host) {
    fail(PFA_EINVAL, "init_cuda: null host");
    return;
  }
  init_core(dev, nx, ny, nm, host->mask_lap[0], kappa, omega, Lmob, D_Cr, D_Nb,
            host->conc_Cr_old[0], host->conc_Nb_old[0], host->phi_del_old[0],
            host->phi_lav_old[0]);
}

void free_cuda(struct CudaData* dev) { free_core(dev); }

void read_out_result(struct CudaData* dev, struct HostData* host, const int nx, const int ny) {
  read_core(dev, host->conc_Cr_new[0], host->conc_Nb_new[0], host->phi_del_new[0],
            host->phi_lav_new[0], nx, ny, true);
}

float nTiles(int domain_size, int tile_loc, int mask_size) {
  return std::ceil(float(domain_size) / float(tile_loc - mask_size + 1));
}

#define PFA_STAGE(call)                                          \
  State* s = lookup(dev);                                        \
  if (!s) return (void)fail(PFA_ESTATE, "unknown CudaData");     \
  if (s->mode != PFA_MODE_COMPAT) return;                        \
  call;

void device_boundaries(struct CudaData* dev, const int, const int, const int, const int, const int) {
  PFA_STAGE(st_boundaries(dev, s))
}
void device_fictitious(struct CudaData* dev, const int, const int, const int, const int, const int) {
  PFA_STAGE(st_fictitious(dev, s))
}
void fictitious_boundaries(struct CudaData* dev, const int, const int, const int, const int,
                           const int) {
  PFA_STAGE(st_fict_boundaries(dev, s))
}
void device_laplacian(struct CudaData* dev, const int, const int, const int, const int, const int,
                      const fp_t dx, const fp_t dy) {
  PFA_STAGE((s->dxy[0] = dx, s->dxy[1] = dy, st_laplacian(dev, s)))
}

// Declared by the reference (src/discretization.cuh:46,67) for its disabled
// variable-mobility form and never defined there.  Here, in compat mode with
// the variable mobility (pfa_set_mobility), they compute the flux
// coefficients and fill their ghost ring; otherwise they return at once.
void device_mobilities(struct CudaData* dev, const int, const int, const int, const int,
                       const int) {
  PFA_STAGE(if (s->varmob) st_mobilities(dev, s))
}
void mobility_boundaries(struct CudaData* dev, const int, const int, const int, const int,
                         const int) {
  PFA_STAGE(if (s->varmob) st_mob_boundaries(dev, s))
}
void device_laplacian_boundaries(struct CudaData* dev, const int, const int, const int, const int,
                                 const int) {
  PFA_STAGE(st_lap_boundaries(dev, s))
}

void device_evolution(struct CudaData* dev, const int, const int, const int, const int, const int,
                      const fp_t alpha, const fp_t dt) {
  State* s = lookup(dev);
  if (!s) return (void)fail(PFA_ESTATE, "device_evolution: unknown CudaData");
  if (s->mode == PFA_MODE_COMPAT)
    st_evolution(dev, s, alpha, dt);
  else
    fused_step(dev, s, alpha, dt);
}

void device_init_prng(struct CudaData* dev, const int, const int, const int, const int, const int) {
  State* s = lookup(dev);
  if (!s) return (void)fail(PFA_ESTATE, "device_init_prng: unknown CudaData");
  s->calls = 0;
  cudaMemsetAsync(s->call_dev, 0, sizeof(unsigned long long), s->st);
}

void device_nucleation(struct CudaData* dev, const int, const int, const int, const int, const int,
                       const fp_t sigma_del, const fp_t sigma_lav, const fp_t unit_a,
                       const fp_t /*ifce_width*/, const fp_t dx, const fp_t dy, const fp_t dz,
                       const fp_t dt) {
  State* s = lookup(dev);
  if (!s) return (void)fail(PFA_ESTATE, "device_nucleation: unknown CudaData");
  nucleate(dev, s, sigma_del, sigma_lav, unit_a, dx, dy, dz, dt);
}

void device_dataviz(struct CudaData* dev, struct HostData* host, const int, const int, const int,
                    const int, const int) {
  dataviz_core(dev, host->conc_Cr_new[0], host->conc_Nb_new[0], host->conc_Ni[0],
               host->phi_del_new[0], host->phi_lav_new[0], host->phi[0]);
}

// ===========================================================================
// extern "C" mirror
extern "C" {

int pfa_last_error(void) { return g_err; }

const char* pfa_error_string(int code) {
  switch (code) {
    case PFA_OK: return "no error";
    case PFA_EINVAL: return "invalid argument or unsupported configuration";
    case PFA_ECUDA: return "CUDA runtime call failed";
    case PFA_ESTATE: return "CudaData not initialised by this library";
    case PFA_EOVERFLOW: return "event buffer overflow";
    case PFA_ENOMEM: return "device allocation failed";
    default: return "unknown error";
  }
}

const char* pfa_last_error_message(void) { return g_msg; }

int pfa_set_device(int device) {
  CK(cudaSetDevice(device));
  return 0;
}

int pfa_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}
void pfa_clear_error(void) {
  g_err = 0;
  g_msg[0] = 0;
}

int pfa_set_mode(struct CudaData* dev, int mode) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_set_mode: unknown CudaData");
  if (mode != PFA_MODE_FUSED && mode != PFA_MODE_COMPAT) return fail(PFA_EINVAL, "pfa_set_mode");
  if (mode == PFA_MODE_COMPAT && s->precision != PFA_FP64)
    return fail(PFA_EINVAL, "compat mode is FP64 only");
  if (mode == PFA_MODE_FUSED && s->varmob && !s->five_point)
    return fail(PFA_EINVAL, "the fused variable-mobility step needs the 5-point mask");
  s->mode = mode;
  return 0;
}

int pfa_set_precision(struct CudaData* dev, int precision) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_set_precision: unknown CudaData");
  if (precision < PFA_FP64 || precision > PFA_FP32_KPHI) return fail(PFA_EINVAL, "pfa_set_precision");
  if (precision != PFA_FP64 && s->mode == PFA_MODE_COMPAT)
    return fail(PFA_EINVAL, "compat mode is FP64 only");
  if (precision != PFA_FP64 && s->varmob && (!s->five_point || !s->zero_sum))
    return fail(PFA_EINVAL, "the FP32 variable-mobility step needs the 5-point mask");
  if (precision != PFA_FP64 && !fp32_records_fit(s->Nx, s->Ny))
    return fail(PFA_EINVAL, "grid above 2^31 records (the FP32 form's 32-bit index)");
  if (precision == s->precision) return 0;
  if (s->f32_live) {
    if (int r = f32_export(dev, s)) return r;
    s->f32_live = false;
  }
  drop_graphs(s);
  s->precision = precision;
  return 0;
}

int pfa_set_mobility(struct CudaData* dev, int model) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_set_mobility: unknown CudaData");
  if (model != PFA_MOBILITY_CONSTANT && model != PFA_MOBILITY_VARIABLE)
    return fail(PFA_EINVAL, "pfa_set_mobility: model");
  if (model == PFA_MOBILITY_VARIABLE) {
    if (s->precision != PFA_FP64 && (!s->five_point || !s->zero_sum))
      return fail(PFA_EINVAL, "the FP32 variable-mobility step needs the 5-point mask");
    if (s->mode == PFA_MODE_FUSED && !s->five_point)
      return fail(PFA_EINVAL, "the fused variable-mobility step needs the 5-point mask");
  }
  s->varmob = model == PFA_MOBILITY_VARIABLE;
  drop_graphs(s);
  return 0;
}

int pfa_set_nucleation(struct CudaData* dev, uint64_t seed, int geometry) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_set_nucleation: unknown CudaData");
  if (geometry != PFA_NUC_REFERENCE_GEOMETRY && geometry != PFA_NUC_FIXED_GEOMETRY)
    return fail(PFA_EINVAL, "pfa_set_nucleation: geometry");
  s->seed = seed;
  s->geometry = geometry;
  s->calls = 0;
  drop_graphs(s);
  CK(cudaMemsetAsync(s->call_dev, 0, sizeof(unsigned long long), s->st));
  return 0;
}

int pfa_set_nucleation_args(struct CudaData* dev, int nuc_interval, double sigma_del,
                            double sigma_lav, double unit_a, double dx, double dy, double dz,
                            double dt_nuc) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_set_nucleation_args: unknown CudaData");
  if (nuc_interval < 0) return fail(PFA_EINVAL, "pfa_set_nucleation_args: interval");
  s->nuc_interval = nuc_interval;
  s->nuc_sigma[0] = sigma_del;
  s->nuc_sigma[1] = sigma_lav;
  s->nuc_unit_a = unit_a;
  s->nuc_d[0] = dx;
  s->nuc_d[1] = dy;
  s->nuc_d[2] = dz;
  s->nuc_dt = dt_nuc;
  s->step_counter = 0;
  drop_graphs(s);
  return 0;
}

int pfa_init_cuda(struct CudaData* dev, int nx, int ny, int nm, const double* mask,
                  const double* kappa, const double* omega, const double* Lmob,
                  const double* D_Cr, const double* D_Nb, const double* conc_Cr,
                  const double* conc_Nb, const double* phi_del, const double* phi_lav) {
  return init_core(dev, nx, ny, nm, mask, kappa, omega, Lmob, D_Cr, D_Nb, conc_Cr, conc_Nb,
                   phi_del, phi_lav);
}

int pfa_free_cuda(struct CudaData* dev) { return free_core(dev); }

int pfa_read_out_result(struct CudaData* dev, double* cr, double* nb, double* pd, double* pl,
                        int nx, int ny) {
  return read_core(dev, cr, nb, pd, pl, nx, ny, true);
}

int pfa_upload_fields(struct CudaData* dev, const double* cr, const double* nb, const double* pd,
                      const double* pl, int nx, int ny) {
  return upload_core(dev, cr, nb, pd, pl, nx, ny, true);
}

int pfa_read_out_result_async(struct CudaData* dev, double* cr, double* nb, double* pd, double* pl,
                              int nx, int ny) {
  return read_core(dev, cr, nb, pd, pl, nx, ny, false);
}

int pfa_upload_fields_async(struct CudaData* dev, const double* cr, const double* nb,
                            const double* pd, const double* pl, int nx, int ny) {
  return upload_core(dev, cr, nb, pd, pl, nx, ny, false);
}

#define PFA_CSTAGE(fn)                                        \
  State* s = lookup(dev);                                     \
  if (!s) return fail(PFA_ESTATE, #fn ": unknown CudaData");  \
  if (s->mode != PFA_MODE_COMPAT) return 0;                   \
  return fn(dev, s);

int pfa_device_boundaries(struct CudaData* dev, int, int, int, int, int) { PFA_CSTAGE(st_boundaries) }
int pfa_device_fictitious(struct CudaData* dev, int, int, int, int, int) { PFA_CSTAGE(st_fictitious) }
int pfa_fictitious_boundaries(struct CudaData* dev, int, int, int, int, int) {
  PFA_CSTAGE(st_fict_boundaries)
}
int pfa_device_laplacian(struct CudaData* dev, int, int, int, int, int, double dx, double dy) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "st_laplacian: unknown CudaData");
  if (s->mode != PFA_MODE_COMPAT) return 0;
  s->dxy[0] = dx;
  s->dxy[1] = dy;
  return st_laplacian(dev, s);
}
int pfa_device_mobilities(struct CudaData* dev, int, int, int, int, int) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_device_mobilities: unknown CudaData");
  if (s->mode != PFA_MODE_COMPAT || !s->varmob) return 0;
  return st_mobilities(dev, s);
}
int pfa_mobility_boundaries(struct CudaData* dev, int, int, int, int, int) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_mobility_boundaries: unknown CudaData");
  if (s->mode != PFA_MODE_COMPAT || !s->varmob) return 0;
  return st_mob_boundaries(dev, s);
}
int pfa_device_laplacian_boundaries(struct CudaData* dev, int, int, int, int, int) {
  PFA_CSTAGE(st_lap_boundaries)
}

int pfa_device_evolution(struct CudaData* dev, int, int, int, int, int, double alpha, double dt) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_device_evolution: unknown CudaData");
  if (s->mode == PFA_MODE_COMPAT) return st_evolution(dev, s, alpha, dt);
  return fused_step(dev, s, alpha, dt);
}

int pfa_device_init_prng(struct CudaData* dev, int nx, int ny, int nm, int bx, int by) {
  if (!lookup(dev)) return fail(PFA_ESTATE, "pfa_device_init_prng: unknown CudaData");
  device_init_prng(dev, nx, ny, nm, bx, by);
  return pfa_last_error() == PFA_OK ? 0 : pfa_last_error();
}

int pfa_device_nucleation(struct CudaData* dev, int, int, int, int, int, double sigma_del,
                          double sigma_lav, double unit_a, double, double dx, double dy, double dz,
                          double dt) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_device_nucleation: unknown CudaData");
  if (int r = nucleate(dev, s, sigma_del, sigma_lav, unit_a, dx, dy, dz, dt)) return r;
  return check_nucleation_status(s);
}

int pfa_device_dataviz(struct CudaData* dev, double* cr, double* nb, double* ni, double* pd,
                       double* pl, double* phi, int nx, int ny) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_device_dataviz: unknown CudaData");
  if (nx != s->nx || ny != s->ny) return fail(PFA_EINVAL, "pfa_device_dataviz: size mismatch");
  return dataviz_core(dev, cr, nb, ni, pd, pl, phi);
}

int pfa_swap(struct CudaData* dev) {
  if (!dev) return fail(PFA_EINVAL, "pfa_swap: null");
  return swap_ptrs(dev);
}

int pfa_run(struct CudaData* dev, int nsteps, double alpha, double dt) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_run: unknown CudaData");
  if (int r = run_core(dev, s, nsteps, alpha, dt)) return r;
  if (s->nuc_interval > 0) return check_nucleation_status(s);
  return 0;
}

int pfa_run_timed(struct CudaData* dev, int nsteps, double alpha, double dt, float* ms) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_run_timed: unknown CudaData");
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaEventRecord(a, s->st));
  const int r = run_core(dev, s, nsteps, alpha, dt);
  CK(cudaEventRecord(b, s->st));
  CK(cudaEventSynchronize(b));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (ms) *ms = t;
  if (r) return r;
  if (s->nuc_interval > 0) return check_nucleation_status(s);
  return 0;
}

// ---- checkpoint / resume ----
int pfa_get_counters(struct CudaData* dev, uint64_t* steps, uint64_t* nucleation_calls) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_get_counters: unknown CudaData");
  if (steps) *steps = s->step_counter;
  if (nucleation_calls) *nucleation_calls = s->calls;
  return 0;
}

int pfa_set_counters(struct CudaData* dev, uint64_t steps, uint64_t nucleation_calls) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_set_counters: unknown CudaData");
  const unsigned long long calls = nucleation_calls;
  CK(cudaMemcpyAsync(s->call_dev, &calls, sizeof(calls), cudaMemcpyHostToDevice, s->st));
  CK(cudaStreamSynchronize(s->st));
  s->step_counter = steps;
  s->calls = nucleation_calls;
  return 0;
}

// bytes of the FP32 form's records: A (16 B) then B (8 B packed, 16 B in
// PFA_FP32_KPHI) for pitch32 x Ny records each
static size_t f32_state_bytes(const State* s) {
  if (s->precision == PFA_FP64) return 0;
  const size_t recs = size_t((s->Nx + 31) / 32) * 32 * s->Ny;
  return recs * 16 + recs * (s->precision == PFA_FP32_KPHI ? 16 : 8);
}

size_t pfa_f32_state_bytes(struct CudaData* dev) {
  State* s = lookup(dev);
  return s ? f32_state_bytes(s) : 0;
}

int pfa_read_f32_state(struct CudaData* dev, void* host, size_t bytes) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_read_f32_state: unknown CudaData");
  if (s->precision == PFA_FP64) return fail(PFA_EINVAL, "pfa_read_f32_state: the handle is FP64");
  if (!host || bytes != f32_state_bytes(s)) return fail(PFA_EINVAL, "pfa_read_f32_state: buffer size");
  if (int r = f32_import(dev, s)) return r;  // the records, from the FP64 fields if not live yet
  const size_t a = size_t(s->pitch32) * s->Ny * 16;
  CK(cudaMemcpyAsync(host, s->recA[s->cur], a, cudaMemcpyDeviceToHost, s->st));
  CK(cudaMemcpyAsync(static_cast<char*>(host) + a, s->recB[s->cur], bytes - a,
                     cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return 0;
}

int pfa_write_f32_state(struct CudaData* dev, const void* host, size_t bytes) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_write_f32_state: unknown CudaData");
  if (s->precision == PFA_FP64) return fail(PFA_EINVAL, "pfa_write_f32_state: the handle is FP64");
  if (!host || bytes != f32_state_bytes(s)) return fail(PFA_EINVAL, "pfa_write_f32_state: buffer size");
  if (int r = ensure_f32(s)) return r;
  const size_t a = size_t(s->pitch32) * s->Ny * 16;
  CK(cudaMemcpyAsync(s->recA[s->cur], host, a, cudaMemcpyHostToDevice, s->st));
  CK(cudaMemcpyAsync(s->recB[s->cur], static_cast<const char*>(host) + a, bytes - a,
                     cudaMemcpyHostToDevice, s->st));
  CK(cudaStreamSynchronize(s->st));
  s->f32_live = true;  // the records are the state now
  return 0;
}

int pfa_sync(struct CudaData* dev) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_sync: unknown CudaData");
  CK(cudaStreamSynchronize(s->st));
  if (dev->str_B) CK(cudaStreamSynchronize(dev->str_B));
  return 0;
}

void* pfa_stream(struct CudaData* dev) {
  State* s = lookup(dev);
  return s ? static_cast<void*>(s->st) : nullptr;
}

int pfa_last_nucleation_events(struct CudaData* dev, int64_t* cells, int32_t* phases, int cap) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_last_nucleation_events: unknown CudaData");
  unsigned n = 0;
  CK(cudaMemcpyAsync(&n, s->ev_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (n > unsigned(kNucCap)) return fail(PFA_EOVERFLOW, "nucleation event buffer overflowed");
  std::vector<NucEvent> ev(n);
  if (n) {
    CK(cudaMemcpyAsync(ev.data(), s->ev, n * sizeof(NucEvent), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
  }
  std::sort(ev.begin(), ev.end(), [](const NucEvent& a, const NucEvent& b) { return a.cell < b.cell; });
  int k = 0;
  for (const auto& e : ev)
    for (int ph = 0; ph < 2; ph++)
      if (e.mask & (1 << ph)) {
        if (k < cap) {
          if (cells) cells[k] = e.cell;
          if (phases) phases[k] = ph;
        }
        k++;
      }
  return k;
}

int pfa_summarize(struct CudaData* dev, double* out) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_summarize: unknown CudaData");
  SumArgs a{};
  if (s->precision != PFA_FP64 && s->f32_live) {
    for (int k = 0; k < 4; k++) a.f[k] = s->recA[s->cur] + k;
    a.comp = s->recB[s->cur];
    a.pack = s->precision == PFA_FP32;
    a.stride = 4;
    a.is_f32 = 1;
    a.compact = 1;
    a.pitch = s->pitch32;
  } else {
    a.f[0] = dev->conc_Cr_old;
    a.f[1] = dev->conc_Nb_old;
    a.f[2] = dev->phi_del_old;
    a.f[3] = dev->phi_lav_old;
    a.pitch = s->nx;
  }
  if (a.stride == 0) a.stride = 1;
  a.Nx = s->Nx;
  a.Ny = s->Ny;
  a.Nz = 1;
  a.partial = s->sum_partial;
  a.out = s->sum_out;
  CK(launch_summarize(a, s->st));
  CK(cudaMemcpyAsync(out, s->sum_out, 5 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return 0;
}

int pfa_summarize_energy(struct CudaData* dev, double dx, double dy, double Omega, double* energy,
                         double* chem_nrg, double* grad_nrg) {
  State* s = lookup(dev);
  if (!s) return fail(PFA_ESTATE, "pfa_summarize_energy: unknown CudaData");
  if (!energy || !(dx > 0.0) || !(dy > 0.0))
    return fail(PFA_EINVAL, "pfa_summarize_energy: needs energy and dx, dy > 0");
  if (int r = f32_export(dev, s)) return r;
  const size_t n = size_t(s->nx) * s->ny;
  double* want[2] = {chem_nrg, grad_nrg};
  for (int k = 0; k < 2; k++)
    if (want[k] && !s->nrg_map[k]) {
      if (alloc_field(&s->nrg_map[k], n)) return PFA_ECUDA;
      CK(cudaMemsetAsync(s->nrg_map[k], 0, n * sizeof(double), s->st));
    }
  EnergyArgs a{};
  a.f[0] = dev->conc_Cr_old;
  a.f[1] = dev->conc_Nb_old;
  a.f[2] = dev->phi_del_old;
  a.f[3] = dev->phi_lav_old;
  a.Nx = s->Nx;
  a.Ny = s->Ny;
  a.Nz = 1;
  a.dxyz[0] = dx;
  a.dxyz[1] = dy;
  a.dxyz[2] = 1.0;
  for (int k = 0; k < 2; k++) {
    a.kappa[k] = s->m.kappa[k];
    a.omega[k] = s->m.omega[k];
  }
  a.Omega = Omega;
  a.chem = chem_nrg ? s->nrg_map[0] : nullptr;
  a.grad = grad_nrg ? s->nrg_map[1] : nullptr;
  a.partial = s->sum_partial;
  a.out = s->sum_out;
  CK(launch_energy(a, s->st));
  CK(cudaMemcpyAsync(energy, s->sum_out, sizeof(double), cudaMemcpyDeviceToHost, s->st));
  for (int k = 0; k < 2; k++)
    if (want[k])
      CK(cudaMemcpyAsync(want[k], s->nrg_map[k], n * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return 0;
}

int pfa_model_params(double dx, double ifce_width, double xcr0, double xnb0, double meshres,
                     int dim, int dt_rule, double* out) {
  if (!out || dx <= 0 || ifce_width <= 0 || (dim != 2 && dim != 3))
    return fail(PFA_EINVAL, "pfa_model_params");
  double Dcr[2] = {model_D(0, 0, xcr0, xnb0), model_D(0, 1, xcr0, xnb0)};
  double Dnb[2] = {model_D(1, 0, xcr0, xnb0), model_D(1, 1, xcr0, xnb0)};
  const double kappa = 3. * kSigma * ifce_width / 2.2;  // src/parameters.h:43-48
  const double omega = 18. * kSigma * kSigma / kappa;
  const double Dnorm = std::sqrt(Dcr[0] * Dcr[0] + Dnb[1] * Dnb[1]);
  const double L = 1.0 * Dnorm / (ifce_width * ifce_width * kRT / kVm);  // src/alloy625.cpp:102-104
  const double rho = model_kks_diffusivity(Dcr, Dnb);
  double target;
  if (dt_rule == 0) {
    const double dtT = (meshres * meshres) / (2.0 * dim * L * kappa);
    const double dtD = (meshres * meshres) / (4.0 * std::fmax(Dcr[0], Dnb[1]));
    target = 0.02 * std::fmin(dtT, dtD);
  } else {
    const double dtT = (dx * dx) / (2.0 * dim * L * kappa);
    const double dtD = (dx * dx) / (2.0 * dim * rho);
    target = 0.5 * std::fmin(dtT, dtD);
  }
  double round_dt = 0.0, roundoff = 4e6;  // src/main.cpp:262-267
  while (round_dt < 1e-20) {
    roundoff *= 10;
    round_dt = std::floor(roundoff * target) / roundoff;
  }
  const double vals[13] = {Dcr[0], Dcr[1], Dnb[0], Dnb[1], kappa, kappa, omega, omega,
                           L,      L,      kOmega, round_dt, rho};
  std::memcpy(out, vals, sizeof(vals));
  return 0;
}

int pfa_model_fast_coef(float* out, int n) {
  if (!out || n < 44) return fail(PFA_EINVAL, "pfa_model_fast_coef");
  FastCoef k;
  model_fast_coef(&k);
  std::memcpy(out, k.den, 6 * sizeof(float));
  std::memcpy(out + 6, k.num, 24 * sizeof(float));
  std::memcpy(out + 30, k.dP, 12 * sizeof(float));
  std::memcpy(out + 42, k.xe_gam, 2 * sizeof(float));
  return 0;
}

int pfa_split_block(const double* in, float* hi, float* c, int n) {
  if (n <= 0 || !in || !hi || !c) return fail(PFA_EINVAL, "pfa_split_block: bad argument");
  double* din = nullptr;
  float* dout = nullptr;
  CK(cudaMalloc(reinterpret_cast<void**>(&din), size_t(n) * 8));
  CK(cudaMalloc(reinterpret_cast<void**>(&dout), size_t(n) * 8));
  CK(cudaMemcpy(din, in, size_t(n) * 8, cudaMemcpyHostToDevice));
  CK(launch_split_block(din, dout, dout + n, n, 0));
  CK(cudaMemcpy(hi, dout, size_t(n) * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(c, dout + n, size_t(n) * 4, cudaMemcpyDeviceToHost));
  cudaFree(din);
  cudaFree(dout);
  return 0;
}

int pfa_philox_block(const uint32_t* ctr, uint64_t key, uint32_t* out, int n) {
  void *dc = nullptr, *dout = nullptr;
  CK(cudaMalloc(&dc, size_t(n) * 16));
  CK(cudaMalloc(&dout, size_t(n) * 16));
  CK(cudaMemcpy(dc, ctr, size_t(n) * 16, cudaMemcpyHostToDevice));
  CK(launch_philox_block(dc, key, dout, n, 0));
  CK(cudaMemcpy(out, dout, size_t(n) * 16, cudaMemcpyDeviceToHost));
  cudaFree(dc);
  cudaFree(dout);
  return 0;
}

}  // extern "C"
