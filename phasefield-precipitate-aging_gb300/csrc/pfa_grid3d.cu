// pfa_grid3d.cu -- 3D grids behind an extern "C" handle API.
//
// The reference is 2D only (src/main.cpp:418-421) and its CudaData has no
// third dimension, so 3D grids get their own handle: create from host fields
// in the ghost-ring layout ((nz x ny x nx) doubles, one ghost cell on every
// face), run n explicit steps (graph-replayed), read back, summarise.  The
// equations are the 2D ones with a 7-point Laplacian (pfa_step3d.cu).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "pfa_gb300.h"
#include "pfa_internal.h"
#include "pfa_kernels.h"
#include "pfa_nucleation.h"
#include "pfa_reduce.h"

namespace pfa {
namespace {

struct Graph {
  int len, nuc_first, cur;
  cudaGraphExec_t exec;
};

struct Grid3D {
  int Nx = 0, Ny = 0, Nz = 0, precision = PFA_FP64;
  ModelConst m{};
  FastCoef fk{};
  cudaStream_t st = nullptr;
  double* f64[2][4] = {};
  float* A[2] = {};
  float* B[2] = {};
  Tma3 tm[2] = {};  // TMA maps of (A[b], B[b])
  int pitch32 = 0;
  double dxyz[3] = {};
  int cur = 0;
  bool f32_live = false;
  double* sum_partial = nullptr;
  double* sum_out = nullptr;
  std::vector<Graph> graphs;
  // nucleation after every step whose index k has k % nuc_interval == 0
  uint64_t seed = 42;
  int nuc_interval = 0;
  double nuc_sigma[2] = {0.13, 0.13}, nuc_unit_a = 0.352e-9, nuc_d[3] = {}, nuc_dt = 0.0;
  uint64_t step_counter = 0;
  NucEvent* ev = nullptr;
  unsigned* ev_count = nullptr;  // [0] events, [1] listed cells
  int* ev_status = nullptr;
  unsigned long long* call_dev = nullptr;  // Philox call counter
  long long* cand = nullptr;               // cells left to the FP64 nucleation decision
  int cand_cap = 0;
  int skip_plane = -1;  // tests only (pfa3d_test_skip_plane): the next run's skipped plane
};

int err(int code, const char* what) {
  std::fprintf(stderr, "pfa_gb300: %s\n", what);
  set_error(code, what);
  return code;
}

int cuda_err(cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  std::fprintf(stderr, "CUDA Runtime Error: %s\n", buf);
  set_error(PFA_ECUDA, buf);
  return PFA_ECUDA;
}

#define CK3(expr)                                          \
  do {                                                     \
    cudaError_t e_ = (expr);                               \
    if (e_ != cudaSuccess) return cuda_err(e_, #expr);     \
  } while (0)

size_t ghost_cells(const Grid3D* g) { return size_t(g->Nx + 2) * (g->Ny + 2) * (g->Nz + 2); }

Conv3DArgs conv(Grid3D* g) {
  Conv3DArgs c{};
  for (int k = 0; k < 4; k++) c.f64[k] = g->f64[0][k];
  c.A = g->A[g->cur];
  c.B = g->B[g->cur];
  c.Nx = g->Nx;
  c.Ny = g->Ny;
  c.Nz = g->Nz;
  c.pitch32 = g->pitch32;
  return c;
}

Step3DArgs step_args(Grid3D* g) {
  Step3DArgs a{};
  a.Nx = g->Nx;
  a.Ny = g->Ny;
  a.Nz = g->Nz;
  a.m = g->m;
  a.k = g->fk;
  const double dt = g->m.dt;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) a.dtD[i][j] = float(dt * g->m.D[i][j]);
  for (int i = 0; i < 2; i++) {
    a.dtL[i] = float(dt * g->m.L[i]);
    a.om2[i] = float(2.0 * g->m.omega[i]);
    a.kap[i] = float(g->m.kappa[i]);
  }
  a.alpha2 = float(2.0 * g->m.alpha);
  for (int i = 0; i < 3; i++) a.idx2f[i] = float(g->m.idx2[i]);
  return a;
}

int step(Grid3D* g) {
  Step3DArgs a = step_args(g);
  const int c = g->cur, n = 1 - c;
  if (g->precision == PFA_FP64) {
    for (int k = 0; k < 4; k++) {
      a.in[k] = g->f64[c][k];
      a.out[k] = g->f64[n][k];
    }
    a.pitch = g->Nx + 2;
    CK3(launch_step3d(a, true, nullptr, g->st));
  } else {
    a.in[0] = g->A[c];
    a.in[1] = g->B[c];
    a.out[0] = g->A[n];
    a.out[1] = g->B[n];
    a.pitch = g->pitch32;
    a.status = g->ev_status;
    a.skip_plane = g->skip_plane;
    CK3(launch_step3d(a, false, &g->tm[c], g->st));
  }
  g->cur = n;
  return 0;
}

int ensure_live(Grid3D* g) {
  if (g->precision == PFA_FP64 || g->f32_live) return 0;
  g->cur = 0;
  CK3(launch_import3d(conv(g), g->st));
  g->f32_live = true;
  return 0;
}

// latest FP64 state in f64[0] (FP64 form: copy if it sits in f64[1])
int sync_f64(Grid3D* g) {
  if (g->precision == PFA_FP64) {
    if (g->cur == 1) {
      const size_t n = ghost_cells(g) * sizeof(double);
      for (int k = 0; k < 4; k++)
        CK3(cudaMemcpyAsync(g->f64[0][k], g->f64[1][k], n, cudaMemcpyDeviceToDevice, g->st));
      g->cur = 0;
    }
    return 0;
  }
  if (g->f32_live) CK3(launch_export3d(conv(g), g->st));
  return 0;
}

// Nucleation on the state after a step (3D form of pfa_nucleation.cu).
int nucleate(Grid3D* g) {
  NucArgs a{};
  const int c = g->cur;
  if (g->precision == PFA_FP64) {
    for (int k = 0; k < 4; k++) a.f[k] = g->f64[c][k];
    a.pitch = g->Nx + 2;
    a.stride = 1;
  } else {
    for (int k = 0; k < 4; k++) a.f[k] = g->A[c] + k;
    a.comp = g->B[c];
    a.pack = 1;
    a.stride = 4;
    a.pitch = g->pitch32;
    a.is_f32 = 1;
    a.compact = 1;
  }
  a.Nx = g->Nx;
  a.Ny = g->Ny;
  a.Nz = g->Nz;
  a.is3d = 1;
  a.sigma[0] = g->nuc_sigma[0];
  a.sigma[1] = g->nuc_sigma[1];
  if (const char* msg =
          nucleation_constants(a, g->nuc_d[0], g->nuc_d[1], g->nuc_d[2], g->nuc_dt, g->nuc_unit_a))
    return err(PFA_EINVAL, msg);
  a.seed = g->seed;
  a.call_ptr = g->call_dev;
  a.events = g->ev;
  a.keys = reinterpret_cast<unsigned long long*>(g->ev + kNucCap);
  a.count = g->ev_count;
  a.status = g->ev_status;
  a.cap = kNucCap;
  a.cand = g->cand;
  a.cand_cap = g->cand_cap;
  CK3(launch_nucleation(a, g->st));
  return 0;
}

// len steps, with a nucleation call after the first when nuc_first
int chunk(Grid3D* g, int len, bool nuc_first) {
  for (int k = 0; k < len; k++) {
    if (int r = step(g)) return r;
    if (k == 0 && nuc_first)
      if (int r = nucleate(g)) return r;
  }
  return 0;
}

// an even number of steps from a captured graph (the ping-pong ends where
// it started)
int graph_chunk(Grid3D* g, int len, bool nuc_first) {
  cudaGraphExec_t exec = nullptr;
  for (auto& e : g->graphs)
    if (e.len == len && e.nuc_first == int(nuc_first) && e.cur == g->cur) exec = e.exec;
  if (!exec) {
    const int cur0 = g->cur;
    cudaGraph_t graph = nullptr;
    CK3(cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal));
    const int r = chunk(g, len, nuc_first);
    const cudaError_t e = cudaStreamEndCapture(g->st, &graph);
    if (r || e != cudaSuccess) {
      // nothing ran: the ping-pong index goes back to the live buffers
      g->cur = cur0;
      if (graph) cudaGraphDestroy(graph);
      return r ? r : cuda_err(e, "cudaStreamEndCapture");
    }
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
      g->cur = cur0;
      return cuda_err(ei, "cudaGraphInstantiate");
    }
    if (g->graphs.size() >= 8) {
      cudaGraphExecDestroy(g->graphs.front().exec);
      g->graphs.erase(g->graphs.begin());
    }
    g->graphs.push_back({len, int(nuc_first), cur0, exec});
    g->cur = cur0;
  }
  CK3(cudaGraphLaunch(exec, g->st));
  return 0;
}

int check_status(Grid3D* g) {
  int st = 0;
  CK3(cudaMemcpyAsync(&st, g->ev_status, sizeof(int), cudaMemcpyDeviceToHost, g->st));
  CK3(cudaStreamSynchronize(g->st));
  if (st) {
    CK3(cudaMemsetAsync(g->ev_status, 0, sizeof(int), g->st));
    if (st == 3) return err(PFA_ECUDA, "3D step: a TMA staging wait gave up (plane copy never landed)");
    if (st == 2) return err(PFA_EINVAL, "nucleation: a nucleus radius exceeded 256 cells (not painted)");
    return err(PFA_EOVERFLOW, "nucleation: more events than the event buffer holds");
  }
  return 0;
}

int run(Grid3D* g, int nsteps) {
  if (int r = ensure_live(g)) return r;
  while (nsteps > 0) {
    int len;
    bool nuc_first = false;
    if (g->nuc_interval > 0) {
      const int phase = int(g->step_counter % uint64_t(g->nuc_interval));
      nuc_first = phase == 0;
      len = std::min(nsteps, g->nuc_interval - phase);
    } else {
      len = std::min(nsteps, 100);
    }
    if (g->skip_plane >= 0) {
      // a test run with a skipped plane goes outside the graphs, which are
      // kept for normal runs
      if (int r = chunk(g, len, nuc_first)) return r;
      g->step_counter += uint64_t(len);
      nsteps -= len;
      continue;
    }
    if (len % 2) {
      // one step outside the graphs, so that they see an even count
      if (int r = chunk(g, 1, nuc_first)) return r;
      g->step_counter += 1;
      nsteps -= 1;
      len -= 1;
      nuc_first = false;
    }
    if (len > 0) {
      if (int r = graph_chunk(g, len, nuc_first)) return r;
      g->step_counter += uint64_t(len);
      nsteps -= len;
    }
  }
  g->skip_plane = -1;
  return g->nuc_interval > 0 ? check_status(g) : 0;
}

}  // namespace
}  // namespace pfa

using namespace pfa;

extern "C" {

size_t pfa3d_footprint(int nx, int ny, int nz, int precision) {
  if (nx < 3 || ny < 3 || nz < 3) return 0;
  const size_t ghost = size_t(nx) * ny * nz;
  const size_t nuc = nucleation_scratch_bytes(size_t(nx - 2) * (ny - 2) * (nz - 2));
  if (precision == PFA_FP64) return 2 * 4 * ghost * sizeof(double) + nuc;
  const size_t recs = size_t((nx - 2 + 31) / 32 * 32) * (ny - 2) * (nz - 2);
  return 4 * ghost * sizeof(double) + 2 * recs * (16 + 8) + nuc;
}

// pfa3d_create's body: the initial fields come from host arrays (src) or
// are built on the device from a recipe (r)
static int create3d(void** handle, int nx, int ny, int nz, const double* params, const double* dxyz,
                    const double* const* src, const pfa_ic_recipe* r, int precision) {
  if (nx < 3 || ny < 3 || nz < 3) return err(PFA_EINVAL, "pfa3d_create: grid smaller than 3^3");
  if (precision != PFA_FP64 && precision != PFA_FP32)
    return err(PFA_EINVAL, "pfa3d_create: 3D grids run in PFA_FP64 or PFA_FP32");
  if (precision == PFA_FP32 && !fp32_records_fit(nx - 2, ny - 2))
    return err(PFA_EINVAL, "pfa3d_create: plane above 2^31 records (the FP32 form's 32-bit index)");
  Grid3D* g = new Grid3D();
  *handle = g;
  g->Nx = nx - 2;
  g->Ny = ny - 2;
  g->Nz = nz - 2;
  g->precision = precision;
  for (int i = 0; i < 2; i++) {
    g->m.D[0][i] = params[i];
    g->m.D[1][i] = params[2 + i];
    g->m.kappa[i] = params[4 + i];
    g->m.omega[i] = params[6 + i];
    g->m.L[i] = params[8 + i];
  }
  g->m.alpha = params[10];
  g->m.dt = params[11];
  for (int i = 0; i < 3; i++) {
    g->dxyz[i] = dxyz[i];
    g->m.idx2[i] = 1.0 / (dxyz[i] * dxyz[i]);
  }
  model_fast_coef(&g->fk);
  static bool ready = false;
  if (!ready) {
    CK3(prepare_step3d());
    CK3(nucleation_setup());
    ready = true;
  }
  CK3(cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking));
  const size_t n = ghost_cells(g);
  const int sets = precision == PFA_FP64 ? 2 : 1;
  for (int b = 0; b < sets; b++)
    for (int k = 0; k < 4; k++) CK3(cudaMalloc(reinterpret_cast<void**>(&g->f64[b][k]), n * sizeof(double)));
  if (r) {
    CK3(launch_ic_fill(*r, g->f64[0], g->st));
  } else {
    for (int k = 0; k < 4; k++)
      CK3(cudaMemcpyAsync(g->f64[0][k], src[k], n * sizeof(double), cudaMemcpyHostToDevice, g->st));
  }
  if (precision == PFA_FP32) {
    g->pitch32 = ((g->Nx + 31) / 32) * 32;
    const size_t recs = size_t(g->pitch32) * g->Ny * g->Nz;
    for (int b = 0; b < 2; b++) {
      CK3(cudaMalloc(reinterpret_cast<void**>(&g->A[b]), recs * 16));
      CK3(cudaMalloc(reinterpret_cast<void**>(&g->B[b]), recs * 8));
      CK3(cudaMemsetAsync(g->A[b], 0, recs * 16, g->st));
      CK3(cudaMemsetAsync(g->B[b], 0, recs * 8, g->st));
      CK3(encode_step3d_maps(&g->tm[b], g->A[b], g->B[b], g->Nx, g->Ny, g->Nz, g->pitch32));
    }
  }
  CK3(cudaMalloc(reinterpret_cast<void**>(&g->sum_partial), sizeof(double) * kSumBlocks * 5));
  CK3(cudaMalloc(reinterpret_cast<void**>(&g->sum_out), sizeof(double) * 5));
  CK3(cudaMalloc(reinterpret_cast<void**>(&g->ev), nucleation_event_bytes()));
  CK3(cudaMalloc(reinterpret_cast<void**>(&g->ev_count), 2 * sizeof(unsigned)));
  g->cand_cap = nucleation_cand_cap(size_t(g->Nx) * g->Ny * g->Nz);
  CK3(cudaMalloc(reinterpret_cast<void**>(&g->cand), sizeof(long long) * size_t(g->cand_cap)));
  CK3(cudaMalloc(reinterpret_cast<void**>(&g->ev_status), sizeof(int)));
  CK3(cudaMalloc(reinterpret_cast<void**>(&g->call_dev), sizeof(unsigned long long)));
  CK3(cudaMemsetAsync(g->ev_count, 0, 2 * sizeof(unsigned), g->st));
  CK3(cudaMemsetAsync(g->ev_status, 0, sizeof(int), g->st));
  CK3(cudaMemsetAsync(g->call_dev, 0, sizeof(unsigned long long), g->st));
  CK3(cudaStreamSynchronize(g->st));
  return 0;
}

int pfa3d_create(void** handle, int nx, int ny, int nz, const double* params, const double* dxyz,
                 const double* conc_Cr, const double* conc_Nb, const double* phi_del,
                 const double* phi_lav, int precision) {
  if (!handle || !params || !dxyz || !conc_Cr || !conc_Nb || !phi_del || !phi_lav)
    return err(PFA_EINVAL, "pfa3d_create: null argument");
  const double* src[4] = {conc_Cr, conc_Nb, phi_del, phi_lav};
  return create3d(handle, nx, ny, nz, params, dxyz, src, nullptr, precision);
}

int pfa3d_create_ic(void** handle, const pfa_ic_recipe* r, const double* params,
                    const double* dxyz, int precision) {
  if (!handle || !params || !dxyz) return err(PFA_EINVAL, "pfa3d_create_ic: null argument");
  if (const char* msg = ic_check(r)) return err(PFA_EINVAL, msg);
  if (r->nz <= 1) return err(PFA_EINVAL, "pfa3d_create_ic: a 3D recipe needs nz > 1");
  return create3d(handle, r->nx + 2, r->ny + 2, r->nz + 2, params, dxyz, nullptr, r, precision);
}

int pfa3d_set_nucleation(void* handle, uint64_t seed, int interval, double sigma_del,
                         double sigma_lav, double unit_a, double dx, double dy, double dz,
                         double dt_nuc) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_set_nucleation: null handle");
  if (interval < 0) return err(PFA_EINVAL, "pfa3d_set_nucleation: negative interval");
  NucArgs a{};
  a.sigma[0] = sigma_del;
  a.sigma[1] = sigma_lav;
  a.is3d = 1;
  a.Nz = g->Nz;
  if (interval > 0)
    if (const char* msg = nucleation_constants(a, dx, dy, dz, dt_nuc, unit_a))
      return err(PFA_EINVAL, msg);
  CK3(cudaStreamSynchronize(g->st));
  for (auto& e : g->graphs) cudaGraphExecDestroy(e.exec);
  g->graphs.clear();
  g->seed = seed;
  g->nuc_interval = interval;
  g->nuc_sigma[0] = sigma_del;
  g->nuc_sigma[1] = sigma_lav;
  g->nuc_unit_a = unit_a;
  g->nuc_d[0] = dx;
  g->nuc_d[1] = dy;
  g->nuc_d[2] = dz;
  g->nuc_dt = dt_nuc;
  g->step_counter = 0;
  CK3(cudaMemsetAsync(g->call_dev, 0, sizeof(unsigned long long), g->st));
  CK3(cudaMemsetAsync(g->ev_count, 0, 2 * sizeof(unsigned), g->st));
  CK3(cudaStreamSynchronize(g->st));
  return 0;
}

int pfa3d_last_nucleation_events(void* handle, int64_t* cells, int32_t* phases, int cap) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_last_nucleation_events: null handle");
  unsigned n = 0;
  CK3(cudaMemcpyAsync(&n, g->ev_count, sizeof(unsigned), cudaMemcpyDeviceToHost, g->st));
  CK3(cudaStreamSynchronize(g->st));
  if (n > unsigned(kNucCap)) return err(PFA_EOVERFLOW, "nucleation event buffer overflowed");
  std::vector<NucEvent> ev(n);
  if (n) {
    CK3(cudaMemcpyAsync(ev.data(), g->ev, n * sizeof(NucEvent), cudaMemcpyDeviceToHost, g->st));
    CK3(cudaStreamSynchronize(g->st));
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

int pfa3d_run(void* handle, int nsteps) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_run: null handle");
  if (nsteps < 0) return err(PFA_EINVAL, "pfa3d_run: negative step count");
  return run(g, nsteps);
}

int pfa3d_run_timed(void* handle, int nsteps, float* ms) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_run_timed: null handle");
  if (int r = ensure_live(g)) return r;
  cudaEvent_t a, b;
  CK3(cudaEventCreate(&a));
  CK3(cudaEventCreate(&b));
  CK3(cudaEventRecord(a, g->st));
  const int r = run(g, nsteps);
  CK3(cudaEventRecord(b, g->st));
  CK3(cudaEventSynchronize(b));
  float t = 0.f;
  CK3(cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (ms) *ms = t;
  return r;
}

int pfa3d_test_skip_plane(void* handle, int plane) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_test_skip_plane: null handle");
  if (g->precision == PFA_FP64) return err(PFA_EINVAL, "pfa3d_test_skip_plane: FP32 form only");
  if (plane < 0 || plane >= g->Nz) return err(PFA_EINVAL, "pfa3d_test_skip_plane: plane");
  g->skip_plane = plane;
  return 0;
}

// ---- checkpoint / resume (as pfa_get_counters ... for CudaData) ----
int pfa3d_get_counters(void* handle, uint64_t* steps, uint64_t* nucleation_calls) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_get_counters: null handle");
  unsigned long long calls = 0;  // the call counter lives on the device
  CK3(cudaMemcpyAsync(&calls, g->call_dev, sizeof(calls), cudaMemcpyDeviceToHost, g->st));
  CK3(cudaStreamSynchronize(g->st));
  if (steps) *steps = g->step_counter;
  if (nucleation_calls) *nucleation_calls = calls;
  return 0;
}

int pfa3d_set_counters(void* handle, uint64_t steps, uint64_t nucleation_calls) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_set_counters: null handle");
  const unsigned long long calls = nucleation_calls;
  CK3(cudaMemcpyAsync(g->call_dev, &calls, sizeof(calls), cudaMemcpyHostToDevice, g->st));
  CK3(cudaStreamSynchronize(g->st));
  g->step_counter = steps;
  return 0;
}

// A (16 B) then packed B (8 B) records, pitch32 x Ny x Nz of each
static size_t f32_state_bytes3(const Grid3D* g) {
  if (g->precision == PFA_FP64) return 0;
  return size_t(g->pitch32) * g->Ny * g->Nz * 24;
}

size_t pfa3d_f32_state_bytes(void* handle) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  return g ? f32_state_bytes3(g) : 0;
}

int pfa3d_read_f32_state(void* handle, void* host, size_t bytes) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_read_f32_state: null handle");
  if (g->precision == PFA_FP64) return err(PFA_EINVAL, "pfa3d_read_f32_state: the grid is FP64");
  if (!host || bytes != f32_state_bytes3(g)) return err(PFA_EINVAL, "pfa3d_read_f32_state: buffer size");
  if (int r = ensure_live(g)) return r;
  const size_t a = size_t(g->pitch32) * g->Ny * g->Nz * 16;
  CK3(cudaMemcpyAsync(host, g->A[g->cur], a, cudaMemcpyDeviceToHost, g->st));
  CK3(cudaMemcpyAsync(static_cast<char*>(host) + a, g->B[g->cur], bytes - a,
                      cudaMemcpyDeviceToHost, g->st));
  return check_status(g);  // waits for the copies
}

int pfa3d_write_f32_state(void* handle, const void* host, size_t bytes) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_write_f32_state: null handle");
  if (g->precision == PFA_FP64) return err(PFA_EINVAL, "pfa3d_write_f32_state: the grid is FP64");
  if (!host || bytes != f32_state_bytes3(g)) return err(PFA_EINVAL, "pfa3d_write_f32_state: buffer size");
  const size_t a = size_t(g->pitch32) * g->Ny * g->Nz * 16;
  CK3(cudaMemcpyAsync(g->A[g->cur], host, a, cudaMemcpyHostToDevice, g->st));
  CK3(cudaMemcpyAsync(g->B[g->cur], static_cast<const char*>(host) + a, bytes - a,
                      cudaMemcpyHostToDevice, g->st));
  CK3(cudaStreamSynchronize(g->st));
  g->f32_live = true;  // the records are the state now
  return 0;
}

int pfa3d_sync(void* handle) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_sync: null handle");
  return check_status(g);
}

// the read-out and the upload, waiting at the end or (wait = 0) only
// enqueued on the handle's stream, which orders everything after them
static int read3d(Grid3D* g, double* const* dst, bool wait) {
  if (int r = sync_f64(g)) return r;
  const size_t n = ghost_cells(g) * sizeof(double);
  for (int k = 0; k < 4; k++)
    if (dst[k]) CK3(cudaMemcpyAsync(dst[k], g->f64[0][k], n, cudaMemcpyDeviceToHost, g->st));
  return wait ? check_status(g) : 0;
}

static int upload3d(Grid3D* g, const double* const* src, bool wait) {
  const size_t n = ghost_cells(g) * sizeof(double);
  for (int k = 0; k < 4; k++)
    CK3(cudaMemcpyAsync(g->f64[0][k], src[k], n, cudaMemcpyHostToDevice, g->st));
  if (wait) CK3(cudaStreamSynchronize(g->st));  // page-locked sources are read asynchronously
  g->cur = 0;
  g->f32_live = false;
  return 0;
}

int pfa3d_read(void* handle, double* conc_Cr, double* conc_Nb, double* phi_del, double* phi_lav) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_read: null handle");
  double* dst[4] = {conc_Cr, conc_Nb, phi_del, phi_lav};
  return read3d(g, dst, true);
}

int pfa3d_read_async(void* handle, double* conc_Cr, double* conc_Nb, double* phi_del,
                     double* phi_lav) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_read_async: null handle");
  double* dst[4] = {conc_Cr, conc_Nb, phi_del, phi_lav};
  return read3d(g, dst, false);
}

int pfa3d_upload(void* handle, const double* conc_Cr, const double* conc_Nb,
                 const double* phi_del, const double* phi_lav) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_upload: null handle");
  if (!conc_Cr || !conc_Nb || !phi_del || !phi_lav) return err(PFA_EINVAL, "pfa3d_upload: null argument");
  const double* src[4] = {conc_Cr, conc_Nb, phi_del, phi_lav};
  return upload3d(g, src, true);
}

int pfa3d_upload_async(void* handle, const double* conc_Cr, const double* conc_Nb,
                       const double* phi_del, const double* phi_lav) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_upload_async: null handle");
  if (!conc_Cr || !conc_Nb || !phi_del || !phi_lav)
    return err(PFA_EINVAL, "pfa3d_upload_async: null argument");
  const double* src[4] = {conc_Cr, conc_Nb, phi_del, phi_lav};
  return upload3d(g, src, false);
}

int pfa3d_summarize(void* handle, double* out) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return err(PFA_ESTATE, "pfa3d_summarize: null handle");
  SumArgs a{};
  if (g->precision == PFA_FP32 && g->f32_live) {
    for (int k = 0; k < 4; k++) a.f[k] = g->A[g->cur] + k;
    a.comp = g->B[g->cur];
    a.pack = 1;
    a.stride = 4;
    a.is_f32 = 1;
    a.compact = 1;
    a.pitch = g->pitch32;
  } else {
    if (int r = sync_f64(g)) return r;
    for (int k = 0; k < 4; k++) a.f[k] = g->f64[0][k];
    a.stride = 1;
    a.pitch = g->Nx + 2;
  }
  a.is3d = 1;
  a.Nx = g->Nx;
  a.Ny = g->Ny;
  a.Nz = g->Nz;
  a.partial = g->sum_partial;
  a.out = g->sum_out;
  CK3(launch_summarize(a, g->st));
  CK3(cudaMemcpyAsync(out, g->sum_out, 5 * sizeof(double), cudaMemcpyDeviceToHost, g->st));
  CK3(cudaStreamSynchronize(g->st));
  return 0;
}

int pfa3d_summarize_energy(void* handle, double Omega, double* energy) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g || !energy) return err(PFA_EINVAL, "pfa3d_summarize_energy: null argument");
  if (int r = sync_f64(g)) return r;
  EnergyArgs a{};
  for (int k = 0; k < 4; k++) a.f[k] = g->f64[0][k];
  a.Nx = g->Nx;
  a.Ny = g->Ny;
  a.Nz = g->Nz;
  a.is3d = 1;
  for (int i = 0; i < 3; i++) a.dxyz[i] = g->dxyz[i];
  for (int k = 0; k < 2; k++) {
    a.kappa[k] = g->m.kappa[k];
    a.omega[k] = g->m.omega[k];
  }
  a.Omega = Omega;
  a.partial = g->sum_partial;
  a.out = g->sum_out;
  CK3(launch_energy(a, g->st));
  CK3(cudaMemcpyAsync(energy, g->sum_out, sizeof(double), cudaMemcpyDeviceToHost, g->st));
  CK3(cudaStreamSynchronize(g->st));
  return 0;
}

int pfa3d_destroy(void* handle) {
  Grid3D* g = static_cast<Grid3D*>(handle);
  if (!g) return 0;
  if (g->st) cudaStreamSynchronize(g->st);
  for (auto& e : g->graphs) cudaGraphExecDestroy(e.exec);
  for (int b = 0; b < 2; b++) {
    for (int k = 0; k < 4; k++) cudaFree(g->f64[b][k]);
    cudaFree(g->A[b]);
    cudaFree(g->B[b]);
  }
  cudaFree(g->sum_partial);
  cudaFree(g->sum_out);
  cudaFree(g->ev);
  cudaFree(g->ev_count);
  cudaFree(g->cand);
  cudaFree(g->ev_status);
  cudaFree(g->call_dev);
  if (g->st) cudaStreamDestroy(g->st);
  delete g;
  return 0;
}

}  // extern "C"
