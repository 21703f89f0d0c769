// pfa_step2d_f32.cu -- the FP32 precision form of the 2D step (sm_103a).
//
// Same step as the FP64 kernel (src/main.cpp:289-305 fused), arithmetic in
// FP32 with every field Kahan-compensated (value = hi - c).  The gamma
// solve is the equilibrium-referenced form (pfa_device.cuh, gamma_u32),
// which keeps FP32 accurate inside precipitates where the plain num / den
// form loses it to cancellation; rows whose phases are all below 1e-5 skip
// the solve (x^gamma = X there).  At 48 bytes per cell the HBM budget leaves
// ~250 instructions per cell, so the kernel is organised for instruction
// economy:
//  * each warp owns a strip of 30 output columns (lanes 1..30; lanes 0 and
//    31 carry the neighbour columns) and streams down a segment of rows; the
//    three rows a 5- or 9-point Laplacian needs live in registers, rotated by
//    a 3x-unrolled loop, so each cell's gamma solve runs once and nothing
//    goes through shared memory;
//  * left / right neighbours come from __shfl_up / __shfl_down (with the
//    9-point mask each row carries its x-difference sums, formed once);
//  * the state is stored as two records per cell -- A = {x_Cr, x_Nb, phi_del,
//    phi_lav} (16 bytes) and B = the four compensations, packed into 16-bit
//    counts (8 bytes, PACK) or as FP32 (16 bytes) -- so a row costs one
//    128-bit and one 64-bit (128-bit) load and store and a single address per
//    lane; records of the row after next are loaded one iteration ahead (the
//    batched kernel stages rows through a per-warp cp.async ring instead).
//
// Record layout: Ny rows of `pitch` records (pitch a multiple of 32), interior
// cell (x, y) at record y * pitch + x, no ghost ring; zero-flux edges come
// from clamped indexing (the mirror the reference's halo fill produces).
#include <cstdint>
#include <type_traits>

#include "pfa_device.cuh"
#include "pfa_kernels.h"

namespace pfa {

using namespace dev;

namespace {

constexpr int kWarps = 4;  // warps (strips) per CTA
constexpr int kCols = 30;  // output columns per warp; lanes 0 and 31 are halo

// The values a neighbour needs: the gamma compositions as deviations
// u = x^gamma - xe_gamma (the variable of the grand-potential difference;
// their Laplacian is that of x^gamma) and the phases.
struct Nb {
  float u1, u2, pd, pl;
};

// With the 9-point mask a row also carries its x-difference sums
// h = (v_w - v) + (v_e - v), formed once per row (two shuffles per field),
// so the diagonal neighbours of the rows above and below cost no shuffles.
struct Nb9 {
  float u1, u2, pd, pl;
  float h1, h2, hd, hl;
};

// With the variable mobility a row also carries each cell's diffusivity
// matrix D(X, Y), scaled by dt / (2 dx^2) (dev::dmat32), for the face sums of
// the divergence.
struct NbV {
  float u1, u2, pd, pl;
  float d00, d01, d10, d11;
};

template <bool NINE, bool VM = false>
using NbT = typename std::conditional<NINE, Nb9,
                                      typename std::conditional<VM, NbV, Nb>::type>::type;

// Compensation record: packed 16-bit counts or four FP32 values.
template <bool PACK>
using CompT = typename std::conditional<PACK, uint2, float4>::type;

template <bool PACK>
struct Raw {
  float4 a;       // x_Cr, x_Nb, phi_del, phi_lav
  CompT<PACK> c;  // Kahan compensations
};

// Per-warp staging ring in shared memory (the batched kernel): rows are
// copied with cp.async kDepth-2 rows ahead of the row being solved, so a warp
// keeps several rows of loads in flight without holding them in registers.
constexpr int kDepth = 4;  // a power of two
template <bool PACK>
struct Ring {
  float4 a[kDepth][32];
  CompT<PACK> c[kDepth][32];
};

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(uint32_t dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <bool PACK>
__device__ __forceinline__ float4 comps(const CompT<PACK>& c) {
  if constexpr (PACK)
    return cq_unpack(c);
  else
    return c;
}

// the composition compensations only (what the gamma solve needs)
template <bool PACK>
__device__ __forceinline__ float2 comps_x(const CompT<PACK>& c) {
  if constexpr (PACK) {
    const float2 h = cq_halves(c.x);
    return make_float2(h.x * kCqXi, h.y * kCqXi);
  } else {
    return make_float2(c.x, c.y);
  }
}

template <bool PACK, bool NINE, bool VM = false>
struct Stream {
  const Step2DArgs& a;
  const float4* A;        // this lane's column, row 0
  const CompT<PACK>* B;
  float4* Ao;
  CompT<PACK>* Bo;
  int Ny, P;
  bool out;  // this lane writes its column

  __device__ __forceinline__ int row(int y) const { return min(max(y, 0), Ny - 1) * P; }

  __device__ __forceinline__ Raw<PACK> load(int off) const {
    return Raw<PACK>{__ldg(A + off), __ldg(B + off)};
  }

  // update row y from its window (up, c, dn); rc = raw centre record
  __device__ __forceinline__ void update(int y, const NbT<NINE, VM>& up, const NbT<NINE, VM>& c,
                                         const NbT<NINE, VM>& dn, const Raw<PACK>& rc) const {
    float lapCr, lapNb, lapD, lapL;
    if constexpr (VM) {
      // variable mobility: lapCr, lapNb hold dt times the divergence of
      // D grad u over the four faces, ((D_n + D_c)(u_n - u_c) summed), the
      // matrices already scaled by dt / (2 dx^2), y faces weighted by qy.
      // Each lane forms the flux through its east face; its west face's is
      // the east flux of the lane to its left (so both cells of a face use
      // the same number, and the x fluxes conserve each component exactly).
      auto dn1 = [](float v) { return __shfl_down_sync(0xffffffffu, v, 1); };
      auto up1 = [](float v) { return __shfl_up_sync(0xffffffffu, v, 1); };
      NbV e;
      e.u1 = dn1(c.u1);
      e.u2 = dn1(c.u2);
      e.d00 = dn1(c.d00);
      e.d01 = dn1(c.d01);
      e.d10 = dn1(c.d10);
      e.d11 = dn1(c.d11);
      // flux of component row (n0 + c0, n1 + c1) into the centre from neighbour n
      auto in = [&](const NbV& n, float n0, float n1, float c0, float c1) {
        return fmaf(n0 + c0, n.u1 - c.u1, (n1 + c1) * (n.u2 - c.u2));
      };
      const float fCr = in(e, e.d00, e.d01, c.d00, c.d01), fNb = in(e, e.d10, e.d11, c.d10, c.d11);
      const float qy = a.vm_qy;
      lapCr = (fCr - up1(fCr)) +
              qy * (in(up, up.d00, up.d01, c.d00, c.d01) + in(dn, dn.d00, dn.d01, c.d00, c.d01));
      lapNb = (fNb - up1(fNb)) +
              qy * (in(up, up.d10, up.d11, c.d10, c.d11) + in(dn, dn.d10, dn.d11, c.d10, c.d11));
      Nb w;
      w.pd = up1(c.pd);
      w.pl = up1(c.pl);
      e.pd = dn1(c.pd);
      e.pl = dn1(c.pl);
      const float idx2 = a.idx2f[0], idy2 = a.idx2f[1];
      auto lap = [&](float vw, float ve, float vn, float vs, float vc) {
        return fmaf((vw - vc) + (ve - vc), idx2, ((vn - vc) + (vs - vc)) * idy2);
      };
      lapD = lap(w.pd, e.pd, up.pd, dn.pd, c.pd);
      lapL = lap(w.pl, e.pl, up.pl, dn.pl, c.pl);
    } else if constexpr (NINE) {
      // sum over the eight neighbours of w (v - v_c): with sy = (v_up - v_c)
      // + (v_dn - v_c) the corners add up to h_up + h_dn + 2 sy; then the
      // sum of the nine weights times the centre value (zero for dx = dy up
      // to rounding; k = that sum times xe_gamma for the deviations u)
      const float ex = a.lap9[0], ey = a.lap9[1], cw = a.lap9[2], sw = a.lap9[3];
      auto lap = [&](float hu, float hc, float hd, float vu, float vc, float vd, float k) {
        const float sy = (vu - vc) + (vd - vc);
        float t = fmaf(sw, vc, k);
        t = fmaf(cw, fmaf(2.0f, sy, hu + hd), t);
        t = fmaf(ey, sy, t);
        return fmaf(ex, hc, t);
      };
      lapCr = lap(up.h1, c.h1, dn.h1, up.u1, c.u1, dn.u1, a.lap9xe[0]);
      lapNb = lap(up.h2, c.h2, dn.h2, up.u2, c.u2, dn.u2, a.lap9xe[1]);
      lapD = lap(up.hd, c.hd, dn.hd, up.pd, c.pd, dn.pd, 0.0f);
      lapL = lap(up.hl, c.hl, dn.hl, up.pl, c.pl, dn.pl, 0.0f);
    } else {
      Nb w, e;
      w.u1 = __shfl_up_sync(0xffffffffu, c.u1, 1);
      w.u2 = __shfl_up_sync(0xffffffffu, c.u2, 1);
      w.pd = __shfl_up_sync(0xffffffffu, c.pd, 1);
      w.pl = __shfl_up_sync(0xffffffffu, c.pl, 1);
      e.u1 = __shfl_down_sync(0xffffffffu, c.u1, 1);
      e.u2 = __shfl_down_sync(0xffffffffu, c.u2, 1);
      e.pd = __shfl_down_sync(0xffffffffu, c.pd, 1);
      e.pl = __shfl_down_sync(0xffffffffu, c.pl, 1);
      const float idx2 = a.idx2f[0], idy2 = a.idx2f[1];
      auto lap = [&](float vw, float ve, float vn, float vs, float vc) {
        const float sx = (vw - vc) + (ve - vc);
        const float sy = (vn - vc) + (vs - vc);
        return fmaf(sx, idx2, sy * idy2);
      };
      lapCr = lap(w.u1, e.u1, up.u1, dn.u1, c.u1);
      lapNb = lap(w.u2, e.u2, up.u2, dn.u2, c.u2);
      lapD = lap(w.pd, e.pd, up.pd, dn.pd, c.pd);
      lapL = lap(w.pl, e.pl, up.pl, dn.pl, c.pl);
    }
    const float4 cc = comps<PACK>(rc.c);
    // Cahn-Hilliard
    const float X = rc.a.x, Y = rc.a.y;
    float ycr, ynb;
    if constexpr (VM) {
      ycr = lapCr - cc.x;
      ynb = lapNb - cc.y;
    } else {
      ycr = fmaf(a.dtD[0][0], lapCr, a.dtD[0][1] * lapNb) - cc.x;
      ynb = fmaf(a.dtD[1][0], lapCr, a.dtD[1][1] * lapNb) - cc.y;
    }
    const float tcr = X + ycr, tnb = Y + ynb;
    // Allen-Cahn
    const FastCoef& K = a.k;
    const float phd = c.pd, phl = c.pl;
    const float dFd = fmaf(-a.kap[0], lapD, dF_local32(phd, phl, quad2(K.dP[0], c.u1, c.u2), a.om2[0], a.alpha2));
    const float dFl = fmaf(-a.kap[1], lapL, dF_local32(phl, phd, quad2(K.dP[1], c.u1, c.u2), a.om2[1], a.alpha2));
    const float yd = fmaf(-a.dtL[0], dFd, -cc.z), td = phd + yd;
    const float yl = fmaf(-a.dtL[1], dFl, -cc.w), tl = phl + yl;
    if (out) {
      const int i = y * P;
      Ao[i] = make_float4(tcr, tnb, td, tl);
      const float ox = (tcr - X) - ycr, oy = (tnb - Y) - ynb;
      const float od = (td - phd) - yd, ol = (tl - phl) - yl;
      if constexpr (PACK)
        Bo[i] = cq_pack(ox, oy, od, ol);
      else
        Bo[i] = make_float4(ox, oy, od, ol);
    }
  }
};

// One warp updates the strip of output columns x0 .. x0+29 over rows
// y0 .. y1-1 of one grid (the unit of work of both the single-grid and the
// batched kernels).  Whole warp; x0 < Nx.  Rows reach the registers either
// directly (one row ahead, !STAGED) or through the warp's staging ring
// (STAGED): the batched kernel's units are short, and the ring's deeper
// prefetch hides the start-up latency each unit pays.
template <bool PACK, bool STAGED, bool NINE = false, bool VM = false>
__device__ __forceinline__ void stream_strip(const Step2DArgs& a, const float4* Ain,
                                             const CompT<PACK>* Bin, float4* Aout,
                                             CompT<PACK>* Bout, int Nx, int Ny, int P, int x0,
                                             int y0, int y1, Ring<PACK>* ring) {
  const int lane = threadIdx.x & 31;
  const int gx = x0 - 1 + lane;  // lanes 0 and 31 hold the neighbour columns
  const int cx = min(max(gx, 0), Nx - 1);
  static_assert(!(STAGED && NINE), "the staged (batched) form has the 5-point mask only");
  static_assert(!(STAGED && VM), "the staged (batched) form has the constant mobility only");
  static_assert(!(NINE && VM), "the variable-mobility form has the 5-point mask only");
  const FastCoef& K = a.k;
  const Stream<PACK, NINE, VM> S{a, Ain + cx, Bin + cx, Aout + cx, Bout + cx,
                             Ny, P, lane >= 1 && lane <= kCols && gx < Nx};
  auto solve_raw = [&](const Raw<PACK>& r) {
    const float2 cxy = comps_x<PACK>(r.c);
    NbT<NINE, VM> n;
    n.pd = r.a.z;
    n.pl = r.a.w;
    // warp-uniform choice: a row of pure gamma needs no solve
    if (__all_sync(0xffffffffu, fmaxf(fabsf(r.a.z), fabsf(r.a.w)) < kBulkPhi))
      gamma_bulk32(K, r.a.x, r.a.y, cxy.x, cxy.y, n.u1, n.u2);
    else
      gamma_u32(K, r.a.x, r.a.y, cxy.x, cxy.y, r.a.z, r.a.w, n.u1, n.u2);
    if constexpr (VM) dmat32(a.vm_pre, r.a.x, r.a.y, n.d00, n.d01, n.d10, n.d11);
    if constexpr (NINE) {
      auto hx = [](float v) {
        return (__shfl_up_sync(0xffffffffu, v, 1) - v) + (__shfl_down_sync(0xffffffffu, v, 1) - v);
      };
      n.h1 = hx(n.u1);
      n.h2 = hx(n.u2);
      n.hd = hx(n.pd);
      n.hl = hx(n.pl);
    }
    return n;
  };
  if constexpr (!STAGED) {
    // window rows y-1, y, y+1 and raw records of rows y, y+1, y+2
    Raw<PACK> r0 = S.load(S.row(y0)), r1 = S.load(S.row(y0 + 1)), r2;
    NbT<NINE, VM> n0 = solve_raw(S.load(S.row(y0 - 1))), n1 = solve_raw(r0), n2;
    // three rows per iteration with rotated roles: no register moves
    int y = y0;
    for (; y + 2 < y1; y += 3) {
      r2 = S.load(S.row(y + 2));
      n2 = solve_raw(r1);
      S.update(y, n0, n1, n2, r0);
      r0 = S.load(S.row(y + 3));
      n0 = solve_raw(r2);
      S.update(y + 1, n1, n2, n0, r1);
      r1 = S.load(S.row(y + 4));
      n1 = solve_raw(r0);
      S.update(y + 2, n2, n0, n1, r2);
    }
    for (; y < y1; y++) {
      r2 = S.load(S.row(y + 2));
      n2 = solve_raw(r1);
      S.update(y, n0, n1, n2, r0);
      n0 = n1;
      n1 = n2;
      r0 = r1;
      r1 = r2;
    }
  } else {
    // ring slot k holds rows y0-1+k, y0-1+k+kDepth, ...; each lane copies and
    // reads back only its own column's records, so the wait needs no warp sync
    const uint32_t sa = uint32_t(__cvta_generic_to_shared(&ring->a[0][lane]));
    const uint32_t sc = uint32_t(__cvta_generic_to_shared(&ring->c[0][lane]));
    constexpr uint32_t kSlotA = 32 * sizeof(float4), kSlotC = 32 * sizeof(CompT<PACK>);
    auto issue = [&](int y, int slot) {
      if (y <= y1) {  // rows past y1 are never read
        const int off = S.row(y);
        cp_async16(sa + slot * kSlotA, S.A + off);
        if constexpr (PACK)
          cp_async8(sc + slot * kSlotC, S.B + off);
        else
          cp_async16(sc + slot * kSlotC, S.B + off);
      }
      cp_commit();  // one group per row (empty past y1): the wait counts stay uniform
    };
    auto fetch = [&](int slot) { return Raw<PACK>{ring->a[slot][lane], ring->c[slot][lane]}; };
#pragma unroll
    for (int k = 0; k < kDepth; k++) issue(y0 - 1 + k, k);
    cp_wait<kDepth - 2>();  // rows y0-1 and y0 have landed
    Nb n0 = solve_raw(fetch(0)), n1 = solve_raw(fetch(1)), n2;
    int s = 0;  // slot of row y-1
    // row y: refill the slot of row y-1 (read for row y-1's update) with row
    // y-1+kDepth, wait for row y+1 (kDepth-2 newer groups stay in flight),
    // solve it, update row y.  Rows up to y1 were all waited for by the last
    // row, so no copy into the ring is pending when the strip ends.
    auto body = [&](int y, const Nb& up, const Nb& c, Nb& dn) {
      issue(y - 1 + kDepth, s);
      s = (s + 1) & (kDepth - 1);
      cp_wait<kDepth - 2>();
      dn = solve_raw(fetch((s + 1) & (kDepth - 1)));
      S.update(y, up, c, dn, fetch(s));
    };
    int y = y0;
    for (; y + 2 < y1; y += 3) {
      body(y, n0, n1, n2);
      body(y + 1, n1, n2, n0);
      body(y + 2, n2, n0, n1);
    }
    for (; y < y1; y++) {
      body(y, n0, n1, n2);
      n0 = n1;
      n1 = n2;
    }
  }
}

// The packed form fits 9 CTAs per SM (56 registers, no spills): the extra
// warps cover load latency (4096^2: 0.1303 ms vs 0.1369 ms at 8); the FP32
// compensation form is faster at 8.  NINE: the 9-point mask (a window of
// eight values per row).
template <bool PACK, bool NINE, bool VM = false>
__global__ void __launch_bounds__(32 * kWarps, VM ? 6 : (PACK && !NINE ? 9 : 8))
    k_stream_f32(Step2DArgs a) {
  const int strip = blockIdx.x * kWarps + (threadIdx.x >> 5);
  const int x0 = strip * kCols;  // first output column of the strip
  if (x0 >= a.Nx) return;        // whole warp leaves together
  const int y0 = blockIdx.y * a.rows;
  stream_strip<PACK, false, NINE, VM>(a, static_cast<const float4*>(a.in[0]),
                            static_cast<const CompT<PACK>*>(a.in[1]),
                            static_cast<float4*>(a.out[0]), static_cast<CompT<PACK>*>(a.out[1]),
                            a.Nx, a.Ny, a.pitch, x0, y0, min(y0 + a.rows, a.Ny), nullptr);
}

// ---- many grids in one launch ----
// Warps claim units (grid, strip, row segment) of the batch's unit table
// through an atomic counter (counter[parity]) until the unit count in
// counter[2] is reached, so a captured launch stays valid while the table's
// contents change.  The launch also zeroes the other parity's counter for the
// next step, which stream order runs after this one.  A persistent launch
// has one CTA per resident slot; the other shape has one warp per unit (and
// leaves the balancing to the block scheduler).  Unit indices come only from
// the counter: ptxas keeps this form within 64 registers without spills.
// Rows are staged through a cp.async ring per warp (12 KB per CTA).
__global__ void __launch_bounds__(32 * kWarps, 8) k_batch_f32(Step2DArgs a, BatchArgs b) {
  const int p = b.parity;
  if (blockIdx.x == 0 && threadIdx.x == 0) b.counter[p ^ 1] = 0;
  const int units = b.counter[2];
  __shared__ Ring<true> ring[kWarps];
  for (;;) {
    int u = 0;
    if ((threadIdx.x & 31) == 0) u = atomicAdd(b.counter + p, 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= units) return;
    const BatchUnit w = b.unit[u];
    const BatchGrid& g = b.grid[w.grid];
    stream_strip<true, true>(a, g.A[p], g.B[p], g.A[p ^ 1], g.B[p ^ 1], g.Nx, g.Ny, g.pitch,
                             w.x0, w.y0, w.y1, &ring[threadIdx.x >> 5]);
  }
}

// ---- layout conversion between the reference's FP64 fields and the form ----
__global__ void k_import_records(ConvArgs a) {
  const int gx = blockIdx.x * blockDim.x + threadIdx.x;
  const int gy = a.y0 + int(blockIdx.y * blockDim.y + threadIdx.y);
  if (gx >= a.Nx || gy >= (a.y1 > 0 ? a.y1 : a.Ny)) return;
  const size_t i64 = size_t(gy + 1) * a.pitch64 + gx + 1;
  const size_t r = size_t(gy) * a.pitch32 + gx;
  float hi[4], c[4];
#pragma unroll
  for (int k = 0; k < 4; k++) split_f64(a.f64[k][i64], hi[k], c[k]);  // value = hi - c
  reinterpret_cast<float4*>(a.A)[r] = make_float4(hi[0], hi[1], hi[2], hi[3]);
  if (a.pack)
    static_cast<uint2*>(a.B)[r] = cq_pack(c[0], c[1], c[2], c[3]);
  else
    static_cast<float4*>(a.B)[r] = make_float4(c[0], c[1], c[2], c[3]);
}

__global__ void k_export_records(ConvArgs a) {
  const int gx = blockIdx.x * blockDim.x + threadIdx.x;
  const int gy = a.y0 + int(blockIdx.y * blockDim.y + threadIdx.y);
  if (gx >= a.Nx || gy >= (a.y1 > 0 ? a.y1 : a.Ny)) return;
  const size_t r = size_t(gy) * a.pitch32 + gx;
  const float4 v = reinterpret_cast<const float4*>(a.A)[r];
  const float4 c = a.pack ? cq_unpack(static_cast<const uint2*>(a.B)[r])
                          : static_cast<const float4*>(a.B)[r];
  const double val[4] = {double(v.x) - double(c.x), double(v.y) - double(c.y),
                         double(v.z) - double(c.z), double(v.w) - double(c.w)};
  const size_t row = size_t(gy + 1) * a.pitch64;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    double* f = a.f64[k];
    f[row + gx + 1] = val[k];
    // ghost ring = mirror of the interior; corners take the diagonal cell
    const bool l = gx == 0, rr = gx == a.Nx - 1, b = gy == 0, t = gy == a.Ny - 1;
    if (l) f[row] = val[k];
    if (rr) f[row + a.Nx + 1] = val[k];
    if (b) {
      f[gx + 1] = val[k];
      if (l) f[0] = val[k];
      if (rr) f[a.Nx + 1] = val[k];
    }
    if (t) {
      const size_t top = size_t(a.Ny + 1) * a.pitch64;
      f[top + gx + 1] = val[k];
      if (l) f[top] = val[k];
      if (rr) f[top + a.Nx + 1] = val[k];
    }
  }
}

// Rows per warp segment: the CTA count should fill whole waves of the
// resident CTAs (a partial last wave idles SMs), while each segment pays two
// extra rows of gamma solves at its ends.
int segment_rows(int Nx, int Ny, int resident) {
  const int nbx = ((Nx + kCols - 1) / kCols + kWarps - 1) / kWarps;
  int best = Ny;
  double best_score = 0.0;
  for (int waves = 1; waves <= 256; waves++) {
    const long long segs = (long long)waves * resident / nbx;
    if (segs < 1) continue;
    const int rows = int((Ny + segs - 1) / segs);
    if (rows < 24 && segs > 1) break;
    const long long used = (long long)nbx * ((Ny + rows - 1) / rows);
    const long long slots = ((used + resident - 1) / resident) * (long long)resident;
    const double score = double(used) / double(slots) / (1.0 + 2.0 / rows);
    if (score > best_score) {
      best_score = score;
      best = rows;
    }
  }
  return best;
}

// resident CTAs: FP32 / packed variants, the batch kernel, the 9-point FP32 / packed
// variants, the variable-mobility FP32 / packed variants
int g_resident[7] = {0, 0, 0, 0, 0, 0, 0};

template <typename K>
cudaError_t query_resident(K kernel, int slot) {
  int dev = 0, sms = 0, per = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 32 * kWarps, 0);
  g_resident[slot] = sms * (per > 0 ? per : 1);
  return e;
}

template <bool PACK, bool NINE, bool VM = false>
cudaError_t launch_stream(Step2DArgs a, cudaStream_t s) {
  const int slot = VM ? 5 + PACK : (NINE ? 3 + PACK : PACK);
  const int resident = g_resident[slot] > 0 ? g_resident[slot] : 152 * 8;
  a.rows = segment_rows(a.Nx, a.Ny, resident);
  const int strips = (a.Nx + kCols - 1) / kCols;
  dim3 grid((strips + kWarps - 1) / kWarps, (a.Ny + a.rows - 1) / a.rows);
  k_stream_f32<PACK, NINE, VM><<<grid, 32 * kWarps, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_step2d_f32(const Step2DArgs& a, cudaStream_t s) {
  if (a.varmob) {
    if (a.nine) return cudaErrorInvalidValue;  // refused by the host before
    return a.full_comp ? launch_stream<false, false, true>(a, s)
                       : launch_stream<true, false, true>(a, s);
  }
  if (a.nine) return a.full_comp ? launch_stream<false, true>(a, s) : launch_stream<true, true>(a, s);
  return a.full_comp ? launch_stream<false, false>(a, s) : launch_stream<true, false>(a, s);
}

// occupancy of the FP32 kernels on the current device (outside any capture)
cudaError_t prepare_step2d_f32() {
  cudaError_t e = query_resident(k_stream_f32<false, false>, 0);
  if (e == cudaSuccess) e = query_resident(k_stream_f32<true, false>, 1);
  if (e == cudaSuccess) e = query_resident(k_batch_f32, 2);
  if (e == cudaSuccess) e = query_resident(k_stream_f32<false, true>, 3);
  if (e == cudaSuccess) e = query_resident(k_stream_f32<true, true>, 4);
  if (e == cudaSuccess) e = query_resident(k_stream_f32<false, false, true>, 5);
  if (e == cudaSuccess) e = query_resident(k_stream_f32<true, false, true>, 6);
  return e;
}

cudaError_t launch_batch_f32(const Step2DArgs& a, const BatchArgs& b, int ctas, cudaStream_t s) {
  const int grid = b.persistent ? ctas : (b.units + kWarps - 1) / kWarps;
  if (grid <= 0) return cudaSuccess;
  k_batch_f32<<<grid, 32 * kWarps, 0, s>>>(a, b);
  return cudaGetLastError();
}

int batch_resident_ctas() { return g_resident[2] > 0 ? g_resident[2] : 152 * 8; }
int batch_warps_per_cta() { return kWarps; }
int batch_strip_cols() { return kCols; }

cudaError_t launch_import_f32(const ConvArgs& a, cudaStream_t s) {
  const int rows = (a.y1 > 0 ? a.y1 : a.Ny) - a.y0;
  if (rows <= 0) return cudaSuccess;
  dim3 block(32, 8);
  dim3 grid((a.Nx + 31) / 32, (rows + 7) / 8);
  k_import_records<<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_export_f32(const ConvArgs& a, cudaStream_t s) {
  const int rows = (a.y1 > 0 ? a.y1 : a.Ny) - a.y0;
  if (rows <= 0) return cudaSuccess;
  dim3 block(32, 8);
  dim3 grid((a.Nx + 31) / 32, (rows + 7) / 8);
  k_export_records<<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pfa
