// pfa_nucleation.cu -- stochastic nucleation of libpfa_gb300 (sm_103a).
//
// The reference's nucleation_kernel (src/discretization.cu:1079-1177) lets
// every thread scan its neighbourhood, draw from a clock-seeded curand XORWOW
// state and paint nuclei into its neighbours' cells while other threads
// read them.  Here the same per-cell physics runs in two deterministic
// phases:
//   1. k_nuc_decide: every interior cell decides on the unmodified fields
//      (neighbourhood scan, driving force g_gam, diffusivities, classical
//      nucleation probability thermo/nucleation.c:30-69) with Philox4x32-10
//      draws keyed by (seed, call counter, cell).  Events are compacted with a
//      warp ballot and one atomic per warp.  The FP64 probability is
//      evaluated only where an FP32 bound cannot exclude an event: if
//      dt dV (J_Cr + J_Nb) < 1e-17 the FP64 P_nuc is 0 or 2^-53 and no draw
//      u >= 2^-53 can fall below it, so skipping such cells changes no
//      decision.  The cells the bound leaves open are listed (same atomic
//      scheme) and
//   1b. k_nuc_fp64 decides them in FP64, 32 listed cells per warp, with the
//      same draws;
//   2. k_nuc_apply: one CTA sorts the events by cell and paints them in that
//      order, delta before laves (embed_OPC_kernel, :1046-1077).
// The event set does not depend on which kernel decided a cell, and the sort
// fixes the painting order.
#include <cmath>
#include <cstdint>

#include "pfa_device.cuh"
#include "pfa_nucleation.cuh"
#include "pfa_nucleation.h"

namespace pfa {

using namespace dev;

namespace {

template <class T>
__global__ void __launch_bounds__(256) k_nuc_decide(NucArgs a) {
  const int gx = blockIdx.x * 32 + (threadIdx.x & 31);
  const int gy = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int nxr = a.Nx + 2, nyr = a.Ny + 2;
  bool need = false;  // the FP32 screen leaves this cell to the FP64 decision
  long long idx = 0;
  size_t s = 0;
  uint4 w = make_uint4(0, 0, 0, 0);
  if (gx < a.Nx && gy < a.Ny) {
    const int x = gx + 1, y = gy + 1, z = a.is3d ? int(blockIdx.z) + 1 : 0;
    idx = ((long long)z * nyr + y) * nxr + x;
    bool clear = true;
    if (a.is3d) {
      // the same scan over a ball; offsets that leave the array along any
      // axis are skipped (no counterpart in the reference)
      const int nzr = a.Nz + 2;
      for (int k = a.scan_lo; k < a.scan_hi && clear; k++)
        for (int j = a.scan_lo; j < a.scan_hi && clear; j++)
          for (int i = a.scan_lo; i < a.scan_hi && clear; i++) {
            if (i * i + j * j + k * k > a.scan_r2) continue;
            const int xx = x + i, yy = y + j, zz = z + k;
            if (xx < 0 || xx >= nxr || yy < 0 || yy >= nyr || zz < 0 || zz >= nzr) continue;
            clear = clear_at<T>(a, stor(a, xx, yy, zz));
          }
    } else {
      // neighbourhood scan of src/discretization.cu:1104-1117 with the
      // reference's double-valued bounds turned into integers on the host
      // (i from (int)(-R) while i < R, i^2 + j^2 < R^2); the reference
      // bounds-checks the linear index nx (y + j) + (x + i), so offsets past
      // a row end wrap onto the next row -- reproduced by normalising (xx, yy)
      for (int i = a.scan_lo; i < a.scan_hi && clear; i++)
        for (int j = a.scan_lo; j < a.scan_hi && clear; j++) {
          if (i * i + j * j > a.scan_r2) continue;
          int xx = x + i, yy = y + j;
          while (xx < 0) {
            xx += nxr;
            yy--;
          }
          while (xx >= nxr) {
            xx -= nxr;
            yy++;
          }
          if (yy < 0 || yy >= nyr) continue;
          clear = clear_at<T>(a, stor(a, xx, yy));
        }
    }
    if (clear) {
      s = stor(a, x, y, z);
      need = nuc_screen(a, float(static_cast<const T*>(a.f[0])[s * a.stride]),
                        float(static_cast<const T*>(a.f[1])[s * a.stride]), idx, w);
    }
  }
  nuc_list_or_decide<T>(a, need, idx, s, w);
}

// The decisions of a call whose neighbourhood scan covers each cell alone
// (R_scan <= 1 cell, as in the reference's geometry): one coalesced load of
// a cell's values, the clear test and the screen.  The pass is bound by
// instruction issue (the screen), not by its 16 B per cell: each thread takes
// kOwnRows cells 8 rows apart and issues their loads before any screen, so
// that four CTAs per SM (64 registers, room for the inlined screen) keep
// enough bytes in flight.
constexpr int kOwnRows = 4;

template <class T>
__global__ void __launch_bounds__(256, 4) k_nuc_decide_own(NucArgs a) {
  const int gx = blockIdx.x * 32 + (threadIdx.x & 31);
  const int gy0 = blockIdx.y * (8 * kOwnRows) + (threadIdx.x >> 5);
  const int z = a.is3d ? int(blockIdx.z) + 1 : 0;
  float v[kOwnRows][4];
#pragma unroll
  for (int r = 0; r < kOwnRows; r++) {
    const int gy = gy0 + 8 * r;
    if (gx < a.Nx && gy < a.Ny) own_values<T>(a, stor(a, gx + 1, gy + 1, z), v[r]);
  }
#pragma unroll
  for (int r = 0; r < kOwnRows; r++) {
    const int gy = gy0 + 8 * r;
    bool need = false;
    long long idx = 0;
    size_t s = 0;
    uint4 w = make_uint4(0, 0, 0, 0);
    if (gx < a.Nx && gy < a.Ny) {
      const int x = gx + 1, y = gy + 1;
      idx = ((long long)z * (a.Ny + 2) + y) * (a.Nx + 2) + x;
      s = stor(a, x, y, z);
      int clear = clear_fp32(v[r][2], v[r][3]);
      if (clear < 0) clear = clear_exact(ldval<T>(a, 2, s), ldval<T>(a, 3, s));
      if (clear) need = nuc_screen(a, v[r][0], v[r][1], idx, w);
    }
    nuc_list_or_decide<T>(a, need, idx, s, w);
  }
}

// The FP64 decisions of the listed cells, 32 per warp.  Consecutive chunks
// of 32 go to different CTAs (chunk c to CTA c mod gridDim.x): a short list
// then spreads over the SMs instead of queueing on one SM's FP64 unit.
template <class T>
__global__ void __launch_bounds__(256) k_nuc_fp64(NucArgs a) {
  const unsigned n = min(a.count[1], unsigned(a.cand_cap));
  const int lane = threadIdx.x & 31;
  const unsigned chunks = (n + 31) / 32;
  const unsigned step = gridDim.x * (blockDim.x >> 5);
  const long long nxr = a.Nx + 2, nyr = a.Ny + 2;
  for (unsigned c = blockIdx.x + gridDim.x * (threadIdx.x >> 5); c < chunks; c += step) {
    const unsigned i = 32 * c + lane;
    bool ev = false;
    NucEvent e;
    if (i < n) {
      const long long idx = a.cand[i];
      const int x = int(idx % nxr);
      const long long t = idx / nxr;
      const int y = int(t % nyr), z = int(t / nyr);
      ev = decide64<T>(a, idx, stor(a, x, y, z), nuc_draw(a, idx), e);
    }
    append_events(a, ev, e);
  }
}

// store v at cell s of field k (and its compensation: value = hi - c)
template <class T>
__device__ __forceinline__ void put(const NucArgs& a, int k, size_t s, double v) {
  static_cast<T*>(a.f[k])[s * a.stride] = T(v);
  comp_set(a, s, k, float(double(T(v)) - v));
}

// embed_OPC_kernel, src/discretization.cu:1046-1077, painted cooperatively
template <class T>
__device__ void paint(const NucArgs& a, const NucEvent& e, int ph) {
  const int nxr = a.Nx + 2;
  const long long ntot = (long long)nxr * (a.Ny + 2);
  const int x = int(e.cell % nxr), y = int(e.cell / nxr);
  const double R = e.r[ph];
  constexpr double xgCr = kXe[0][0], xgNb = kXe[0][1];
  constexpr double xdCr = kXe[1][0], xdNb = kXe[1][1], xlCr = kXe[2][0], xlNb = kXe[2][1];
  const double parCr = ph == 0 ? xdCr : xlCr, parNb = ph == 0 ? xdNb : xlNb;
  const int lo = int(-R);
  int hi = lo;
  while (double(hi) < R) hi++;  // loop bound of `for (i = -R; i < R; i++)`
  const int w = hi - lo;
  if (w <= 0) return;  // (uniform over the block: every thread paints the same event)
  // depletion radii: one thread evaluates them (an FP64 divide and square
  // root per thread of the block would cost ~50 us per event on this part's
  // FP64 unit) and shares them
  __shared__ double s_rd[2];
  if (threadIdx.x == 0) {
    s_rd[0] = R * sqrt((parCr - e.xcr) / (e.xcr - xgCr));
    s_rd[1] = R * sqrt((parNb - e.xnb) / (e.xnb - xgNb));
  }
  __syncthreads();
  const double RdCr = s_rd[0], RdNb = s_rd[1];
  if (a.is3d) {
    // spheres (no counterpart in the reference): offsets that leave the
    // array along any axis are skipped
    const int nyr = a.Ny + 2, nzr = a.Nz + 2;
    const int x3 = int(e.cell % nxr), y3 = int((e.cell / nxr) % nyr);
    const int z3 = int(e.cell / ((long long)nxr * nyr));
    const long long n3 = (long long)w * w * w;
    for (long long t = threadIdx.x; t < n3; t += blockDim.x) {
      const int i = lo + int(t % w), j = lo + int((t / w) % w), k = lo + int(t / ((long long)w * w));
      const int xx = x3 + i, yy = y3 + j, zz = z3 + k;
      if (xx < 0 || xx >= nxr || yy < 0 || yy >= nyr || zz < 0 || zz >= nzr) continue;
      // the FP32 form keeps no ghost ring: a nucleus never paints one there
      if (a.compact && (xx == 0 || yy == 0 || zz == 0 || xx == nxr - 1 || yy == nyr - 1 ||
                        zz == nzr - 1))
        continue;
      const size_t s = stor(a, xx, yy, zz);
      const double r = sqrt(double(i * i + j * j + k * k));
      if (r <= R) {
        put<T>(a, 0, s, parCr);
        put<T>(a, 1, s, parNb);
        put<T>(a, 2 + ph, s, 1.0);
      } else {
        if (r <= RdCr) put<T>(a, 0, s, xgCr);
        if (r <= RdNb) put<T>(a, 1, s, xgNb);
      }
    }
    return;
  }
  const long long n = (long long)w * w;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = lo + int(t / w), j = lo + int(t % w);
    const long long idn = (long long)nxr * (y + j) + (x + i);
    if (idn < 0 || idn >= ntot) continue;
    const int yy = int(idn / nxr), xx = int(idn % nxr);
    // the FP32 form keeps no ghost ring: a nucleus never paints one there
    if (a.compact && (xx == 0 || yy == 0 || xx == nxr - 1 || yy == a.Ny + 1)) continue;
    const size_t s = stor(a, xx, yy);
    const double r = sqrt(double(i * i + j * j));
    if (r <= R) {
      put<T>(a, 0, s, parCr);
      put<T>(a, 1, s, parNb);
      put<T>(a, 2 + ph, s, 1.0);
    } else {
      if (r <= RdCr) put<T>(a, 0, s, xgCr);
      if (r <= RdNb) put<T>(a, 1, s, xgNb);
    }
  }
}

// paint() of an event whose nuclei lie within its own cell (radius < 1
// cell: the box is the cell, at distance 0 <= R): the precipitate's
// composition and phase, delta before laves
template <class T>
__device__ void paint_own(const NucArgs& a, const NucEvent& e) {
  const long long nxr = a.Nx + 2, nyr = a.Ny + 2;
  const int x = int(e.cell % nxr);
  const long long t = e.cell / nxr;
  const int y = int(t % nyr), z = int(t / nyr);
  const size_t s = stor(a, x, y, a.is3d ? z : 0);
  constexpr double xdCr = kXe[1][0], xdNb = kXe[1][1], xlCr = kXe[2][0], xlNb = kXe[2][1];
  for (int ph = 0; ph < 2; ph++)
    if (e.mask & (1 << ph)) {
      put<T>(a, 0, s, ph == 0 ? xdCr : xlCr);
      put<T>(a, 1, s, ph == 0 ? xdNb : xlNb);
      put<T>(a, 2 + ph, s, 1.0);
    }
}

template <class T>
__global__ void __launch_bounds__(1024) k_nuc_apply(NucArgs a) {
  const unsigned n = *a.count;
  __syncthreads();
  // the decision kernel of this call has read the counter: advance it
  if (threadIdx.x == 0) *a.call_ptr += 1ull;
  if (n == 0) return;
  if (n > unsigned(a.cap)) {
    if (threadIdx.x == 0) *a.status = 1;  // overflow: nothing painted
    return;
  }
  // When every nucleus of the call has a radius below one cell, paint's box
  // is the event's own cell, and events come from distinct cells: they touch
  // disjoint cells, so they are painted at once, one thread each.
  bool own = true;
  for (unsigned t = threadIdx.x; t < n; t += blockDim.x) {
    const NucEvent& e = a.events[t];
    for (int ph = 0; ph < 2; ph++)
      if ((e.mask & (1 << ph)) && !(e.r[ph] < 1.0)) own = false;
  }
  if (__syncthreads_and(own)) {
    for (unsigned t = threadIdx.x; t < n; t += blockDim.x) paint_own<T>(a, a.events[t]);
    return;
  }
  // bitonic sort of (cell, event index) keys, ascending, in the global
  // scratch beside the events (no shared memory, so the launch asks for no
  // large shared allocation on the calls, most of them, with few events)
  unsigned long long* key = a.keys;
  unsigned m = 1;
  while (m < n) m <<= 1;
  for (unsigned t = threadIdx.x; t < m; t += blockDim.x)
    key[t] = t < n ? ((unsigned long long)a.events[t].cell << kNucIdxBits) | t : ~0ull;
  __syncthreads();
  for (unsigned k = 2; k <= m; k <<= 1)
    for (unsigned j = k >> 1; j > 0; j >>= 1) {
      for (unsigned t = threadIdx.x; t < m; t += blockDim.x) {
        const unsigned p = t ^ j;
        if (p > t) {
          const unsigned long long u = key[t], v = key[p];
          const bool up = (t & k) == 0;
          if ((u > v) == up) {
            key[t] = v;
            key[p] = u;
          }
        }
      }
      __syncthreads();
    }
  for (unsigned q = 0; q < n; q++) {
    const NucEvent e = a.events[key[q] & ((1ull << kNucIdxBits) - 1)];
    for (int ph = 0; ph < 2; ph++) {
      if (e.mask & (1 << ph)) paint<T>(a, e, ph);
      __syncthreads();
    }
  }
}

}  // namespace

cudaError_t launch_nucleation(const NucArgs& a, cudaStream_t s) {
  cudaError_t err = cudaMemsetAsync(a.count, 0, 2 * sizeof(unsigned), s);
  if (err != cudaSuccess) return err;
  dim3 grid((a.Nx + 31) / 32, (a.Ny + 7) / 8, a.is3d ? a.Nz : 1);
  const bool own = a.scan_lo == 0 && a.scan_hi == 1;  // the scan covers each cell alone
  // grid-stride over the FP64 list (its length is on the device): a CTA per SM
  const int fp64_blocks = 152;
  // k_nuc_decide_own: 32 x (8 kOwnRows) cells per CTA
  const dim3 grid_own(grid.x, (a.Ny + 8 * kOwnRows - 1) / (8 * kOwnRows), grid.z);
  if (a.is_f32) {
    if (own)
      k_nuc_decide_own<float><<<grid_own, 256, 0, s>>>(a);
    else
      k_nuc_decide<float><<<grid, 256, 0, s>>>(a);
    k_nuc_fp64<float><<<fp64_blocks, 256, 0, s>>>(a);
    k_nuc_apply<float><<<1, 1024, 0, s>>>(a);
  } else {
    if (own)
      k_nuc_decide_own<double><<<grid_own, 256, 0, s>>>(a);
    else
      k_nuc_decide<double><<<grid, 256, 0, s>>>(a);
    k_nuc_fp64<double><<<fp64_blocks, 256, 0, s>>>(a);
    k_nuc_apply<double><<<1, 1024, 0, s>>>(a);
  }
  return cudaGetLastError();
}

const char* nucleation_constants(NucArgs& a, double dx, double dy, double dz, double dt,
                                 double unit_a) {
  const bool ok = std::isfinite(dx) && std::isfinite(dy) && std::isfinite(dz) &&
                  std::isfinite(dt) && std::isfinite(unit_a) && dx > 0 && dy > 0 && dz > 0 &&
                  dt > 0 && unit_a > 0 && std::isfinite(a.sigma[0]) && std::isfinite(a.sigma[1]);
  if (!ok) return "nucleation: spacing, time and lattice must be finite and > 0";
  if (!(1.75e-9 / dx <= kNucMaxScan))
    return "nucleation: neighbourhood scan radius 1.75 nm / dx exceeds 64 cells";
  if (a.is3d && a.Nz > 65535) return "nucleation: more than 65535 planes";
  a.dx = dx;
  a.dV = dx * dy * dz;
  a.Vatom = 0.25 * unit_a * unit_a * unit_a;
  a.n_gam = a.dV / a.Vatom;
  a.dt = dt;
  a.R_scan = 1.75e-9 / dx;
  a.ln_dtdV = std::log(dt * a.dV);
  a.ln_ngam = std::log(a.n_gam);
  // the reference's loop `for (int i = -R; i < R; i++)` with the test
  // i*i + j*j < R*R, in integers: lo = (int)(-R), hi = first int >= R,
  // r2 = largest int < R*R
  const double R = a.R_scan;
  a.scan_lo = int(-R);
  int hi = a.scan_lo;
  while (double(hi) < R) hi++;
  a.scan_hi = hi;
  const double R2 = R * R;
  long long m = (long long)std::floor(R2);
  if (double(m) >= R2) m--;  // strictly below R^2
  a.scan_r2 = int(m);
  // constants of the FP32 screen (ln_z_tier1, ln_z_tier2):
  // ln k1_k = lnK + ln(D_kk x_k) (ln(dt dV) folded in), k2 = C2 / dG^2
  for (int ph = 0; ph < 2; ph++) {
    const double sg = a.sigma[ph], s3 = sg * sg * sg;
    const double a4 = std::pow(kLatticeConst, 4);
    const double lnG = std::log(16.0 * kPi * s3 / 3.0);                        // G* dG^2
    const double lnZ = std::log(a.Vatom / (8.0 * kPi * std::sqrt(kKT * s3)));  // Zeldovich / dG^2
    const double lnK = std::log(3.0) + lnG - std::log(sg) - std::log(a4) + lnZ + a.ln_ngam +
                       a.ln_dtdV;
    a.lnK[ph] = float(lnK);
    // |D_kk| <= 3 x 1.5e-20 x 2.5e6 exp(max e); two terms at most twice one
    a.lnC1[ph] = float(lnK + std::log(3.0 * 1.5e-20 * 2.5e6) + std::log(2.0));
    a.C2[ph] = float(16.0 * kPi * s3 / (3.0 * kKT));
  }
  return nullptr;
}

cudaError_t nucleation_setup() { return cudaSuccess; }

// The FP32-form split exposed for its test (one block of doubles).
__global__ void k_split_block(const double* in, float* hi, float* c, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) split_f64(in[i], hi[i], c[i]);
}

cudaError_t launch_split_block(const double* in, float* hi, float* c, int n, cudaStream_t s) {
  k_split_block<<<(n + 255) / 256, 256, 0, s>>>(in, hi, c, n);
  return cudaGetLastError();
}

// Philox exposed for the generator test (one block of counters).
__global__ void k_philox_block(const uint4* ctr, uint2 key, uint4* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = philox4x32_10(ctr[i], key);
}

cudaError_t launch_philox_block(const void* ctr, uint64_t key, void* out, int n, cudaStream_t s) {
  k_philox_block<<<(n + 255) / 256, 256, 0, s>>>(static_cast<const uint4*>(ctr),
                                                  make_uint2(uint32_t(key), uint32_t(key >> 32)),
                                                  static_cast<uint4*>(out), n);
  return cudaGetLastError();
}

}  // namespace pfa
