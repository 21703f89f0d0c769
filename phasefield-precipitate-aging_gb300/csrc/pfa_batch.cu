// pfa_batch.cu -- many independent 2D grids stepped together.
//
// The reference steps one grid per process (src/main.cpp:285-321).  A batch
// holds any number of 2D grids of different sizes that share one parameter
// set, in the FP32 precision form (packed compensations), and advances all of
// them with one launch per time step: the grids' warp strips x row segments
// form one table of units of work that a persistent kernel drains through an
// atomic counter (or that a one-warp-per-unit launch covers).  Multi-step runs
// replay captured CUDA graphs.  Grids join and leave between runs
// (continuous batching): each owns one block of a fixed device arena (first
// fit, coalescing free list), so the batch's device footprint is decided when
// it is created and a grid that does not fit is refused with PFA_ENOMEM.
//
// Every cell's update reads only its own grid's records, and a unit's result
// does not depend on how rows are split into segments, so a grid advances
// bit-for-bit the same alone, in any batch, and as a single-grid handle.
//
// Host transfers do not wait for the GPU.  The FP64 fields of adds and reads
// pass through a staging ring in device memory, copied on two copy streams
// (host to device, device to host); the conversions to and from the FP32
// records run on a high-priority stream of their own, ordered against the
// step stream with events.  So one batch's copies run while another batch's
// persistent step kernel holds the SMs, and its conversions are dispatched
// ahead of the next step launch.  A stream that writes a ring region first
// waits for the event of the region's last reader (a stream wait, not a host
// wait); an import into an arena block waits for the steps enqueued before
// the latest removal, which may still read a freed block.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <vector>

#include "pfa_gb300.h"
#include "pfa_internal.h"
#include "pfa_kernels.h"
#include "pfa_reduce.h"

namespace pfa {
namespace {

constexpr size_t kAlign = 256;

struct Slot {
  bool live = false;
  int Nx = 0, Ny = 0, pitch = 0;
  size_t off = 0, bytes = 0;  // block in the arena
};

// a region of the staging ring and the event after its last use
struct RingEntry {
  size_t begin, end;
  cudaEvent_t done;
};

struct BGraph {
  int len, parity, grid;
  unsigned long long version;
  cudaGraphExec_t exec;
};

struct Batch {
  cudaStream_t st = nullptr;
  Step2DArgs a{};  // shared constants
  char* arena = nullptr;
  size_t cap = 0, used = 0;
  std::map<size_t, size_t> free_;  // offset -> size
  std::vector<Slot> slots;
  int cur = 0;
  BatchGrid* d_grid = nullptr;
  int grid_cap = 0;
  BatchUnit* d_unit = nullptr;
  int unit_cap = 0;
  int* d_counter = nullptr;  // counters of parity 0 / 1, unit count
  int units = 0;
  bool dirty = true;
  int rows = 64;         // rows per segment
  int persistent = 1;    // persistent launch (else one warp per unit)
  int ctas = 0;          // CTAs of a persistent launch (0 = all resident)
  unsigned long long version = 1;  // bumps when the device tables move
  std::vector<BGraph> graphs;
  cudaStream_t up = nullptr, down = nullptr;  // host -> device / device -> host copies
  cudaStream_t cv = nullptr;                  // conversions (high priority)
  cudaEvent_t removed = nullptr;              // the step stream at the latest removal
  bool fence = false;                         // a removal since the last import
  char* ring = nullptr;                       // FP64 staging of adds and reads
  size_t ring_cap = 0, ring_head = 0;
  std::deque<RingEntry> ring_q;               // regions in use, in allocation order
  std::vector<cudaEvent_t> ev_pool;
  double* sum_partial = nullptr;
  double* sum_out = nullptr;
};

int fail(int code, const char* what) {
  std::fprintf(stderr, "pfa_gb300: %s\n", what);
  set_error(code, what);
  return code;
}

int fail_cuda(cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  std::fprintf(stderr, "CUDA Runtime Error: %s\n", buf);
  set_error(PFA_ECUDA, buf);
  return PFA_ECUDA;
}

#define CKB(expr)                                        \
  do {                                                   \
    cudaError_t e_ = (expr);                             \
    if (e_ != cudaSuccess) return fail_cuda(e_, #expr);  \
  } while (0)

size_t block_bytes(int Nx, int Ny) {
  const size_t pitch = size_t((Nx + 31) / 32) * 32;
  const size_t b = pitch * size_t(Ny) * 48;  // A (16 B) + B (8 B), two parities
  return (b + kAlign - 1) / kAlign * kAlign;
}

// record buffers of a slot: A0, A1, B0, B1 inside its block
BatchGrid grid_entry(const Batch* b, const Slot& s) {
  BatchGrid g{};
  const size_t recs = size_t(s.pitch) * s.Ny;
  char* base = b->arena + s.off;
  g.A[0] = reinterpret_cast<float4*>(base);
  g.A[1] = reinterpret_cast<float4*>(base + recs * 16);
  g.B[0] = reinterpret_cast<uint2*>(base + recs * 32);
  g.B[1] = reinterpret_cast<uint2*>(base + recs * 40);
  g.Nx = s.Nx;
  g.Ny = s.Ny;
  g.pitch = s.pitch;
  return g;
}

bool arena_alloc(Batch* b, size_t bytes, size_t* off) {
  for (auto it = b->free_.begin(); it != b->free_.end(); ++it) {
    if (it->second < bytes) continue;
    *off = it->first;
    const size_t rest = it->second - bytes;
    const size_t at = it->first + bytes;
    b->free_.erase(it);
    if (rest) b->free_[at] = rest;
    b->used += bytes;
    return true;
  }
  return false;
}

void arena_free(Batch* b, size_t off, size_t bytes) {
  b->used -= bytes;
  auto it = b->free_.emplace(off, bytes).first;
  auto nx = std::next(it);
  if (nx != b->free_.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    b->free_.erase(nx);
  }
  if (it != b->free_.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      b->free_.erase(it);
    }
  }
}

// The unit table for the current members and segment length: every grid's
// rows are split into equal segments of at most `rows`; units are ordered by
// decreasing length so that the counter hands out the long ones first.
void make_units(const Batch* b, int rows, std::vector<BatchUnit>* out) {
  const int cols = batch_strip_cols();
  out->clear();
  for (int i = 0; i < int(b->slots.size()); i++) {
    const Slot& s = b->slots[i];
    if (!s.live) continue;
    const int segs = std::max(1, (s.Ny + rows - 1) / rows);
    const int r = (s.Ny + segs - 1) / segs;
    for (int x0 = 0; x0 < s.Nx; x0 += cols)
      for (int y0 = 0; y0 < s.Ny; y0 += r) out->push_back({i, x0, y0, std::min(s.Ny, y0 + r)});
  }
  std::stable_sort(out->begin(), out->end(), [](const BatchUnit& p, const BatchUnit& q) {
    return p.y1 - p.y0 > q.y1 - q.y0;
  });
}

int upload_tables(Batch* b, int rows) {
  std::vector<BatchGrid> grids(b->slots.size());
  for (size_t i = 0; i < b->slots.size(); i++)
    if (b->slots[i].live) grids[i] = grid_entry(b, b->slots[i]);
  std::vector<BatchUnit> units;
  make_units(b, rows, &units);
  if (int(grids.size()) > b->grid_cap) {
    cudaStreamSynchronize(b->st);
    cudaFree(b->d_grid);
    b->d_grid = nullptr;
    b->grid_cap = std::max<int>(64, int(grids.size()) * 2);
    CKB(cudaMalloc(reinterpret_cast<void**>(&b->d_grid), sizeof(BatchGrid) * b->grid_cap));
    b->version++;
  }
  if (int(units.size()) > b->unit_cap) {
    cudaStreamSynchronize(b->st);
    cudaFree(b->d_unit);
    b->d_unit = nullptr;
    b->unit_cap = std::max<int>(4096, int(units.size()) * 2);
    CKB(cudaMalloc(reinterpret_cast<void**>(&b->d_unit), sizeof(BatchUnit) * b->unit_cap));
    b->version++;
  }
  // the copies are stream-ordered after every launch already enqueued
  if (!grids.empty())
    CKB(cudaMemcpyAsync(b->d_grid, grids.data(), sizeof(BatchGrid) * grids.size(),
                        cudaMemcpyHostToDevice, b->st));
  if (!units.empty())
    CKB(cudaMemcpyAsync(b->d_unit, units.data(), sizeof(BatchUnit) * units.size(),
                        cudaMemcpyHostToDevice, b->st));
  b->units = int(units.size());
  const int counters[3] = {0, 0, b->units};
  CKB(cudaMemcpyAsync(b->d_counter, counters, sizeof(counters), cudaMemcpyHostToDevice, b->st));
  // no host wait: copies from pageable host memory are staged before
  // cudaMemcpyAsync returns, and the launches that read the tables follow
  // them on the stream
  return 0;
}

int refresh(Batch* b) {
  if (!b->dirty) return 0;
  if (int r = upload_tables(b, b->rows)) return r;
  b->dirty = false;
  return 0;
}

int persistent_ctas(const Batch* b) {
  const int res = batch_resident_ctas();
  const int need = (b->units + batch_warps_per_cta() - 1) / batch_warps_per_cta();
  const int c = b->ctas > 0 ? b->ctas : res;
  return std::max(1, std::min(c, need));
}

int launch(Batch* b, int parity) {
  BatchArgs ba{};
  ba.grid = b->d_grid;
  ba.unit = b->d_unit;
  ba.counter = b->d_counter;
  ba.units = b->units;
  ba.parity = parity;
  ba.persistent = b->persistent;
  CKB(launch_batch_f32(b->a, ba, persistent_ctas(b), b->st));
  return 0;
}

int run(Batch* b, int nsteps) {
  if (int r = refresh(b)) return r;
  if (b->units == 0) return 0;
  while (nsteps > 0) {
    if (nsteps == 1) {
      if (int r = launch(b, b->cur)) return r;
      b->cur ^= 1;
      return 0;
    }
    const int len = std::min(nsteps - nsteps % 2, 100);
    // a persistent launch reads the unit count from the device; the other
    // mode's grid size is the unit count
    const int gsize = b->persistent ? persistent_ctas(b) : -b->units;
    cudaGraphExec_t exec = nullptr;
    for (auto& g : b->graphs)
      if (g.len == len && g.parity == b->cur && g.grid == gsize && g.version == b->version)
        exec = g.exec;
    if (!exec) {
      // graphs of moved tables are not replayed again; keep at most 8
      for (auto& g : b->graphs)
        if (g.version != b->version) cudaGraphExecDestroy(g.exec);
      b->graphs.erase(std::remove_if(b->graphs.begin(), b->graphs.end(),
                                     [&](const BGraph& g) { return g.version != b->version; }),
                      b->graphs.end());
      if (b->graphs.size() >= 8) {
        cudaGraphExecDestroy(b->graphs.front().exec);
        b->graphs.erase(b->graphs.begin());
      }
      cudaGraph_t graph;
      CKB(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
      int r = 0;
      for (int k = 0; k < len && !r; k++) r = launch(b, b->cur ^ (k & 1));
      const cudaError_t e = cudaStreamEndCapture(b->st, &graph);
      if (r) return r;
      if (e != cudaSuccess) return fail_cuda(e, "cudaStreamEndCapture");
      CKB(cudaGraphInstantiate(&exec, graph, 0));
      cudaGraphDestroy(graph);
      b->graphs.push_back({len, b->cur, gsize, b->version, exec});
    }
    CKB(cudaGraphLaunch(exec, b->st));
    nsteps -= len;  // even: the parity is back where it was
  }
  return 0;
}

cudaError_t take_event(Batch* b, cudaEvent_t* ev) {
  if (!b->ev_pool.empty()) {
    *ev = b->ev_pool.back();
    b->ev_pool.pop_back();
    return cudaSuccess;
  }
  return cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
}

// `waiter` waits (on the device) for everything enqueued so far on `from`
int order_after(Batch* b, cudaStream_t waiter, cudaStream_t from) {
  cudaEvent_t ev;
  CKB(take_event(b, &ev));
  CKB(cudaEventRecord(ev, from));
  CKB(cudaStreamWaitEvent(waiter, ev, 0));
  b->ev_pool.push_back(ev);  // the wait holds the state it was enqueued with
  return 0;
}

// n bytes of the staging ring for a region that `writer` fills first: the
// writer waits for the last readers of the bytes it overwrites
int ring_take(Batch* b, size_t n, cudaStream_t writer, size_t* off) {
  n = (n + kAlign - 1) / kAlign * kAlign;
  // drop the regions whose last use has completed (oldest first)
  while (!b->ring_q.empty()) {
    const cudaError_t q = cudaEventQuery(b->ring_q.front().done);
    if (q == cudaErrorNotReady) {
      // not an error: clear it if the query left it as the thread's last
      // error, and leave any other pending error for its own check
      if (cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();
      break;
    }
    CKB(q);
    b->ev_pool.push_back(b->ring_q.front().done);
    b->ring_q.pop_front();
  }
  if (n > b->ring_cap) {  // grow: rare; drain every stream first
    for (cudaStream_t x : {b->up, b->cv, b->st, b->down}) CKB(cudaStreamSynchronize(x));
    for (auto& e : b->ring_q) b->ev_pool.push_back(e.done);
    b->ring_q.clear();
    cudaFree(b->ring);
    b->ring = nullptr;
    b->ring_cap = std::max(n, 2 * b->ring_cap);
    CKB(cudaMalloc(reinterpret_cast<void**>(&b->ring), b->ring_cap));
    b->ring_head = 0;
  }
  size_t at = b->ring_head;
  if (at + n > b->ring_cap) at = 0;
  for (auto it = b->ring_q.begin(); it != b->ring_q.end();) {
    if (it->begin < at + n && at < it->end) {
      CKB(cudaStreamWaitEvent(writer, it->done, 0));
      b->ev_pool.push_back(it->done);
      it = b->ring_q.erase(it);
    } else {
      ++it;
    }
  }
  b->ring_head = at + n;
  *off = at;
  return 0;
}

// the region [off, off + n) is free once `last` has done what is enqueued on it
int ring_release(Batch* b, size_t off, size_t n, cudaStream_t last) {
  n = (n + kAlign - 1) / kAlign * kAlign;
  cudaEvent_t ev;
  CKB(take_event(b, &ev));
  CKB(cudaEventRecord(ev, last));
  b->ring_q.push_back({off, off + n, ev});
  return 0;
}

// the four FP64 fields of an nx x ny grid in the ring region at off
void ring_fields(const Batch* b, size_t off, size_t cells, double* f[4]) {
  for (int k = 0; k < 4; k++) f[k] = reinterpret_cast<double*>(b->ring + off) + k * cells;
}

ConvArgs conv(Batch* b, const Slot& s, double* const f64[4]) {
  const BatchGrid g = grid_entry(b, s);
  ConvArgs c{};
  for (int k = 0; k < 4; k++) c.f64[k] = f64[k];
  c.A = reinterpret_cast<float*>(g.A[b->cur]);
  c.B = g.B[b->cur];
  c.pack = 1;
  c.Nx = s.Nx;
  c.Ny = s.Ny;
  c.pitch64 = s.Nx + 2;
  c.pitch32 = s.pitch;
  return c;
}

// the conversion stream waits for the steps enqueued before the latest
// removal (an arena block freed there may be handed to the grid imported next)
int await_removals(Batch* b) {
  if (!b->fence) return 0;
  CKB(cudaStreamWaitEvent(b->cv, b->removed, 0));
  b->fence = false;
  return 0;
}

// the export of a live slot into the ring and its copies to host arrays
// (null: skipped) on the device-to-host stream; no host wait
int read_async(Batch* b, const Slot& s, double* const dst[4]) {
  const size_t cells = size_t(s.Nx + 2) * (s.Ny + 2), n = 4 * cells * sizeof(double);
  size_t off = 0;
  if (int r = ring_take(b, n, b->cv, &off)) return r;
  double* f[4];
  ring_fields(b, off, cells, f);
  if (int r = order_after(b, b->cv, b->st)) return r;  // after the runs enqueued so far
  CKB(launch_export_f32(conv(b, s, f), b->cv));
  if (int r = order_after(b, b->down, b->cv)) return r;
  for (int k = 0; k < 4; k++)
    if (dst[k])
      CKB(cudaMemcpyAsync(dst[k], f[k], cells * sizeof(double), cudaMemcpyDeviceToHost, b->down));
  return ring_release(b, off, n, b->down);
}

Batch* get(void* h) { return static_cast<Batch*>(h); }

const Slot* live_slot(Batch* b, int slot) {
  if (!b || slot < 0 || slot >= int(b->slots.size()) || !b->slots[slot].live) return nullptr;
  return &b->slots[slot];
}

// A slot for an nx x ny grid (ghost-ring sizes) in the arena; its records
// are filled by the caller (an import from FP64 fields in the staging ring).
int place(Batch* b, int nx, int ny, int* id_out) {
  Slot s;
  s.Nx = nx - 2;
  s.Ny = ny - 2;
  s.pitch = (s.Nx + 31) / 32 * 32;
  s.bytes = block_bytes(s.Nx, s.Ny);
  if (!arena_alloc(b, s.bytes, &s.off)) {
    set_error(PFA_ENOMEM, "pfa_batch_add: the grid does not fit in the batch arena");
    return PFA_ENOMEM;  // admission refusal: not printed
  }
  s.live = true;
  int id = -1;
  for (int i = 0; i < int(b->slots.size()); i++)
    if (!b->slots[i].live) {
      id = i;
      break;
    }
  if (id < 0) {
    id = int(b->slots.size());
    b->slots.push_back(s);
  } else {
    b->slots[id] = s;
  }
  *id_out = id;
  return 0;
}

}  // namespace
}  // namespace pfa

using namespace pfa;

extern "C" {

size_t pfa_batch_footprint(int nx, int ny) {
  if (nx < 3 || ny < 3) return 0;
  return block_bytes(nx - 2, ny - 2);
}

int pfa_batch_create(void** handle, const double* params, const double* dxy, size_t arena_bytes) {
  if (!handle || !params || !dxy) return fail(PFA_EINVAL, "pfa_batch_create: null argument");
  if (arena_bytes < kAlign) return fail(PFA_EINVAL, "pfa_batch_create: arena smaller than 256 bytes");
  static std::once_flag ready;
  static cudaError_t ready_err = cudaSuccess;
  std::call_once(ready, [] { ready_err = prepare_step2d_f32(); });
  CKB(ready_err);
  Batch* b = new Batch();
  *handle = b;
  Step2DArgs& a = b->a;
  ModelConst& m = a.m;
  for (int i = 0; i < 2; i++) {
    m.D[0][i] = params[i];
    m.D[1][i] = params[2 + i];
    m.kappa[i] = params[4 + i];
    m.omega[i] = params[6 + i];
    m.L[i] = params[8 + i];
  }
  m.alpha = params[10];
  m.dt = params[11];
  m.idx2[0] = 1.0 / (dxy[0] * dxy[0]);
  m.idx2[1] = 1.0 / (dxy[1] * dxy[1]);
  model_fast_coef(&a.k);
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) a.dtD[i][j] = float(m.dt * m.D[i][j]);
  for (int i = 0; i < 2; i++) {
    a.dtL[i] = float(m.dt * m.L[i]);
    a.om2[i] = float(2.0 * m.omega[i]);
    a.kap[i] = float(m.kappa[i]);
  }
  a.alpha2 = float(2.0 * m.alpha);
  a.idx2f[0] = float(m.idx2[0]);
  a.idx2f[1] = float(m.idx2[1]);
  b->cap = arena_bytes / kAlign * kAlign;
  CKB(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
  CKB(cudaStreamCreateWithFlags(&b->up, cudaStreamNonBlocking));
  CKB(cudaStreamCreateWithFlags(&b->down, cudaStreamNonBlocking));
  int lo = 0, hi = 0;
  CKB(cudaDeviceGetStreamPriorityRange(&lo, &hi));
  CKB(cudaStreamCreateWithPriority(&b->cv, cudaStreamNonBlocking, hi));
  CKB(cudaEventCreateWithFlags(&b->removed, cudaEventDisableTiming));
  // staging ring: the arena's size within [16 MiB, 8 GiB]; it grows for a
  // larger single grid
  b->ring_cap = std::min<size_t>(std::max<size_t>(b->cap, size_t(16) << 20), size_t(8) << 30);
  CKB(cudaMalloc(reinterpret_cast<void**>(&b->ring), b->ring_cap));
  CKB(cudaMalloc(reinterpret_cast<void**>(&b->arena), b->cap));
  b->free_[0] = b->cap;
  CKB(cudaMalloc(reinterpret_cast<void**>(&b->d_counter), 3 * sizeof(int)));
  CKB(cudaMemsetAsync(b->d_counter, 0, 3 * sizeof(int), b->st));
  CKB(cudaMalloc(reinterpret_cast<void**>(&b->sum_partial), sizeof(double) * kSumBlocks * 5));
  CKB(cudaMalloc(reinterpret_cast<void**>(&b->sum_out), sizeof(double) * 5));
  CKB(cudaStreamSynchronize(b->st));
  return 0;
}

int pfa_batch_add(void* handle, int nx, int ny, const double* conc_Cr, const double* conc_Nb,
                  const double* phi_del, const double* phi_lav, int* slot) {
  Batch* b = get(handle);
  if (!b) return fail(PFA_ESTATE, "pfa_batch_add: null handle");
  if (!conc_Cr || !conc_Nb || !phi_del || !phi_lav || !slot)
    return fail(PFA_EINVAL, "pfa_batch_add: null argument");
  if (nx < 3 || ny < 3) return fail(PFA_EINVAL, "pfa_batch_add: grid smaller than 3x3");
  if (!fp32_records_fit(nx - 2, ny - 2))
    return fail(PFA_EINVAL, "pfa_batch_add: grid above 2^31 records (the FP32 form's 32-bit index)");
  int id = -1;
  if (int r = place(b, nx, ny, &id)) return r;
  const size_t cells = size_t(nx) * ny, n = 4 * cells * sizeof(double);
  size_t off = 0;
  if (int r = ring_take(b, n, b->up, &off)) return r;
  double* f[4];
  ring_fields(b, off, cells, f);
  const double* src[4] = {conc_Cr, conc_Nb, phi_del, phi_lav};
  for (int k = 0; k < 4; k++)
    CKB(cudaMemcpyAsync(f[k], src[k], cells * sizeof(double), cudaMemcpyHostToDevice, b->up));
  if (int r = order_after(b, b->cv, b->up)) return r;
  if (int r = await_removals(b)) return r;
  CKB(launch_import_f32(conv(b, b->slots[id], f), b->cv));
  if (int r = order_after(b, b->st, b->cv)) return r;  // the steps read the block
  if (int r = ring_release(b, off, n, b->cv)) return r;
  b->dirty = true;
  *slot = id;
  return 0;
}

int pfa_batch_add_ic(void* handle, const pfa_ic_recipe* r, int* slot) {
  Batch* b = get(handle);
  if (!b) return fail(PFA_ESTATE, "pfa_batch_add_ic: null handle");
  if (!slot) return fail(PFA_EINVAL, "pfa_batch_add_ic: null argument");
  if (const char* msg = ic_check(r)) return fail(PFA_EINVAL, msg);
  if (r->nz > 1) return fail(PFA_EINVAL, "pfa_batch_add_ic: the batch holds 2D grids (nz <= 1)");
  const int nx = r->nx + 2, ny = r->ny + 2;
  if (nx < 3 || ny < 3) return fail(PFA_EINVAL, "pfa_batch_add_ic: grid smaller than 3x3");
  if (!fp32_records_fit(nx - 2, ny - 2))
    return fail(PFA_EINVAL, "pfa_batch_add_ic: grid above 2^31 records (the FP32 form's 32-bit index)");
  int id = -1;
  if (int e = place(b, nx, ny, &id)) return e;
  const size_t cells = size_t(nx) * ny, n = 4 * cells * sizeof(double);
  size_t off = 0;
  if (int e = ring_take(b, n, b->cv, &off)) return e;
  double* f[4];
  ring_fields(b, off, cells, f);
  if (int e = await_removals(b)) return e;
  CKB(launch_ic_fill(*r, f, b->cv));
  CKB(launch_import_f32(conv(b, b->slots[id], f), b->cv));
  if (int e = order_after(b, b->st, b->cv)) return e;  // the steps read the block
  if (int e = ring_release(b, off, n, b->cv)) return e;
  b->dirty = true;
  *slot = id;
  return 0;
}

int pfa_batch_remove(void* handle, int slot) {
  Batch* b = get(handle);
  const Slot* s = live_slot(b, slot);
  if (!s) return fail(PFA_EINVAL, "pfa_batch_remove: no such grid");
  // launches already enqueued may still read the block: the next import
  // (which may reuse it) waits for them
  CKB(cudaEventRecord(b->removed, b->st));
  b->fence = true;
  arena_free(b, s->off, s->bytes);
  b->slots[slot].live = false;
  b->dirty = true;
  return 0;
}

int pfa_batch_read(void* handle, int slot, double* conc_Cr, double* conc_Nb, double* phi_del,
                   double* phi_lav) {
  Batch* b = get(handle);
  const Slot* s = live_slot(b, slot);
  if (!s) return fail(PFA_EINVAL, "pfa_batch_read: no such grid");
  double* const dst[4] = {conc_Cr, conc_Nb, phi_del, phi_lav};
  if (int r = read_async(b, *s, dst)) return r;
  CKB(cudaStreamSynchronize(b->down));
  return 0;
}

int pfa_batch_read_async(void* handle, int slot, double* conc_Cr, double* conc_Nb,
                         double* phi_del, double* phi_lav) {
  Batch* b = get(handle);
  const Slot* s = live_slot(b, slot);
  if (!s) return fail(PFA_EINVAL, "pfa_batch_read_async: no such grid");
  double* const dst[4] = {conc_Cr, conc_Nb, phi_del, phi_lav};
  return read_async(b, *s, dst);
}

int pfa_batch_run(void* handle, int nsteps) {
  Batch* b = get(handle);
  if (!b) return fail(PFA_ESTATE, "pfa_batch_run: null handle");
  if (nsteps < 0) return fail(PFA_EINVAL, "pfa_batch_run: negative step count");
  return run(b, nsteps);
}

int pfa_batch_run_timed(void* handle, int nsteps, float* ms) {
  Batch* b = get(handle);
  if (!b) return fail(PFA_ESTATE, "pfa_batch_run_timed: null handle");
  if (int r = refresh(b)) return r;
  cudaEvent_t e0, e1;
  CKB(cudaEventCreate(&e0));
  CKB(cudaEventCreate(&e1));
  CKB(cudaEventRecord(e0, b->st));
  const int r = run(b, nsteps);
  CKB(cudaEventRecord(e1, b->st));
  CKB(cudaEventSynchronize(e1));
  float t = 0.f;
  CKB(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ms) *ms = t;
  return r;
}

int pfa_batch_sync(void* handle) {
  Batch* b = get(handle);
  if (!b) return fail(PFA_ESTATE, "pfa_batch_sync: null handle");
  for (cudaStream_t x : {b->up, b->cv, b->st, b->down}) CKB(cudaStreamSynchronize(x));
  return 0;
}

int pfa_batch_set_launch(void* handle, int rows, int persistent, int ctas) {
  Batch* b = get(handle);
  if (!b) return fail(PFA_ESTATE, "pfa_batch_set_launch: null handle");
  if (rows < 1 || ctas < 0) return fail(PFA_EINVAL, "pfa_batch_set_launch: rows >= 1, ctas >= 0");
  b->rows = rows;
  b->persistent = persistent ? 1 : 0;
  b->ctas = ctas;
  b->dirty = true;
  return 0;
}

int pfa_batch_get_launch(void* handle, int* rows, int* persistent, int* ctas, int* units) {
  Batch* b = get(handle);
  if (!b) return fail(PFA_ESTATE, "pfa_batch_get_launch: null handle");
  if (int r = refresh(b)) return r;
  if (rows) *rows = b->rows;
  if (persistent) *persistent = b->persistent;
  if (ctas) *ctas = b->persistent ? persistent_ctas(b) : (b->units + batch_warps_per_cta() - 1) / batch_warps_per_cta();
  if (units) *units = b->units;
  return 0;
}

int pfa_batch_tune(void* handle, int reps, float* best_ms) {
  Batch* b = get(handle);
  if (!b) return fail(PFA_ESTATE, "pfa_batch_tune: null handle");
  if (reps < 1) reps = 10;
  static const int kRows[] = {16, 24, 32, 48, 64, 96, 128, 256, 1 << 30};
  float best = -1.f;
  int best_rows = b->rows, best_pers = b->persistent;
  cudaEvent_t e0, e1;
  CKB(cudaEventCreate(&e0));
  CKB(cudaEventCreate(&e1));
  for (int pers = 0; pers < 2; pers++) {
    for (int rows : kRows) {
      if (int r = upload_tables(b, rows)) return r;
      if (b->units == 0) break;
      b->persistent = pers;
      // cur -> cur ^ 1 every time: the grids' state does not advance
      for (int k = 0; k < reps + 2; k++) {
        if (k == 2) CKB(cudaEventRecord(e0, b->st));
        CKB(cudaMemsetAsync(b->d_counter, 0, 2 * sizeof(int), b->st));
        if (int r = launch(b, b->cur)) return r;
      }
      CKB(cudaEventRecord(e1, b->st));
      CKB(cudaEventSynchronize(e1));
      float t = 0.f;
      CKB(cudaEventElapsedTime(&t, e0, e1));
      t /= reps;
      if (best < 0.f || t < best) {
        best = t;
        best_rows = rows;
        best_pers = pers;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->rows = best_rows;
  b->persistent = best_pers;
  b->dirty = true;
  if (int r = refresh(b)) return r;
  if (best_ms) *best_ms = best;
  return 0;
}

int pfa_batch_summarize(void* handle, int slot, double* out) {
  Batch* b = get(handle);
  const Slot* s = live_slot(b, slot);
  if (!s || !out) return fail(PFA_EINVAL, "pfa_batch_summarize: no such grid");
  const BatchGrid g = grid_entry(b, *s);
  SumArgs a{};
  const float* A = reinterpret_cast<const float*>(g.A[b->cur]);
  for (int k = 0; k < 4; k++) a.f[k] = A + k;
  a.comp = g.B[b->cur];
  a.pack = 1;
  a.stride = 4;
  a.is_f32 = 1;
  a.compact = 1;
  a.pitch = s->pitch;
  a.Nx = s->Nx;
  a.Ny = s->Ny;
  a.Nz = 1;
  a.partial = b->sum_partial;
  a.out = b->sum_out;
  CKB(launch_summarize(a, b->st));
  CKB(cudaMemcpyAsync(out, b->sum_out, 5 * sizeof(double), cudaMemcpyDeviceToHost, b->st));
  CKB(cudaStreamSynchronize(b->st));
  return 0;
}

int pfa_batch_info(void* handle, int* grids, size_t* used_bytes, size_t* arena_bytes) {
  Batch* b = get(handle);
  if (!b) return fail(PFA_ESTATE, "pfa_batch_info: null handle");
  int n = 0;
  for (const Slot& s : b->slots) n += s.live;
  if (grids) *grids = n;
  if (used_bytes) *used_bytes = b->used;
  if (arena_bytes) *arena_bytes = b->cap;
  return 0;
}

void* pfa_batch_stream(void* handle) {
  Batch* b = get(handle);
  return b ? static_cast<void*>(b->st) : nullptr;
}

int pfa_batch_destroy(void* handle) {
  Batch* b = get(handle);
  if (!b) return 0;
  for (cudaStream_t x : {b->up, b->cv, b->st, b->down})
    if (x) cudaStreamSynchronize(x);
  if (b->removed) cudaEventDestroy(b->removed);
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
  for (auto& e : b->ring_q) cudaEventDestroy(e.done);
  for (cudaEvent_t e : b->ev_pool) cudaEventDestroy(e);
  cudaFree(b->ring);
  cudaFree(b->arena);
  cudaFree(b->d_grid);
  cudaFree(b->d_unit);
  cudaFree(b->d_counter);
  cudaFree(b->sum_partial);
  cudaFree(b->sum_out);
  for (cudaStream_t x : {b->up, b->cv, b->st, b->down})
    if (x) cudaStreamDestroy(x);
  delete b;
  return 0;
}

}  // extern "C"
