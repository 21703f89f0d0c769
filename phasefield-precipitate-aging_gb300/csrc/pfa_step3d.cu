// pfa_step3d.cu -- 3D step with the 7-point Laplacian (sm_103a).
//
// The reference supports 2D only (src/main.cpp:418-421); this extends its
// equations unchanged to a 7-point stencil with six-face zero-flux ghost
// fill.  Two kernels stream along z:
//   k_stream3d_f64: plain FP64, the reference's formulas, ghost-ring layout
//        ((Nz+2) planes of (Ny+2) rows of Nx+2 doubles, one array per field);
//        a CTA of 16 warps covers 30 x-columns (lanes 1..30) by 14 y-rows
//        (warps 1..14); lanes 0 / 31 and warps 0 / 15 carry the neighbour
//        columns and rows.  x-neighbours come from shuffles, y-neighbours
//        from planes published in shared memory, z-neighbours from a
//        three-plane register window rotated by a 3x-unrolled loop, one
//        barrier per plane.
//   k_stream3d_f32: the precision form (FP32 arithmetic, every field
//        Kahan-compensated, the equilibrium-referenced gamma solve) on
//        interior-only records (pfa_step2d_f32.cu): A = float4 {x_Cr, x_Nb,
//        phi_del, phi_lav}, B = the four compensations as packed 16-bit
//        counts (uint2); tiles of 32 x 13 output cells, records staged by
//        TMA, described below.
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <type_traits>

#include "pfa_device.cuh"
#include "pfa_kernels.h"
#include "pfa_tma.cuh"

namespace pfa {

using namespace dev;

namespace {

constexpr int kW = 16;  // FP64: warps per CTA (y-rows including the 2 halo rows)
constexpr int kRowsOut = kW - 2;
constexpr int kCols = 30;  // FP64: output columns per warp

template <class R>
struct Nb3 {
  R gcr, gnb, pd, pl;
};

// FP64: gcr / gnb are x^gamma; FP32: the deviations u = x^gamma - xe_gamma
template <class R>
struct Raw3 {
  R x, y, pd, pl;
  uint2 cq;  // FP32: packed Kahan compensations
};

// FP64 store of the interior cell (x, y, z) and of every ghost cell whose
// nearest interior cell it is (the six-face fill; edges and corners take the
// nearest interior cell).
__device__ __forceinline__ void store64(double* f, const Step3DArgs& a, int x, int y, int z,
                                        double v) {
  int xs[3] = {x, 0, 0}, ys[3] = {y, 0, 0}, zs[3] = {z, 0, 0};
  int nx = 1, ny = 1, nz = 1;
  if (x == 0) xs[nx++] = -1;
  if (x == a.Nx - 1) xs[nx++] = a.Nx;
  if (y == 0) ys[ny++] = -1;
  if (y == a.Ny - 1) ys[ny++] = a.Ny;
  if (z == 0) zs[nz++] = -1;
  if (z == a.Nz - 1) zs[nz++] = a.Nz;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++)
        f[((long long)(zs[k] + 1) * (a.Ny + 2) + (ys[j] + 1)) * a.pitch + (xs[i] + 1)] = v;
}

// One thread's column of the FP64 kernel.
struct S64 {
  const Step3DArgs& a;
  int cx, cy;  // clamped column / row of this thread
  bool out;    // this thread owns an output column and row

  __device__ __forceinline__ long long cell(int z) const {
    const int zz = min(max(z, 0), a.Nz - 1);
    return ((long long)(zz + 1) * (a.Ny + 2) + (cy + 1)) * a.pitch + (cx + 1);
  }

  __device__ __forceinline__ Raw3<double> load(int z) const {
    const long long i = cell(z);
    Raw3<double> r;
    r.x = __ldg(static_cast<const double*>(a.in[0]) + i);
    r.y = __ldg(static_cast<const double*>(a.in[1]) + i);
    r.pd = __ldg(static_cast<const double*>(a.in[2]) + i);
    r.pl = __ldg(static_cast<const double*>(a.in[3]) + i);
    r.cq = make_uint2(0u, 0u);
    return r;
  }

  // gamma solve of one cell
  __device__ __forceinline__ Nb3<double> solve(const Raw3<double>& r) const {
    const double pD = p64(r.pd), pL = p64(r.pl), pG = 1.0 - pD - pL;
    Poly64 m;
    poly64(pD, pG, pL, m);
    return Nb3<double>{fict64<0, 0>(r.x, r.y, m), fict64<0, 1>(r.x, r.y, m), r.pd, r.pl};
  }

  // update plane z of this thread's column from the window (up, c, dn)
  __device__ __forceinline__ void update(int z, const Nb3<double>& up, const Nb3<double>& c,
                                         const Nb3<double>& dn, const Raw3<double>& rc,
                                         Nb3<double> (*sh)[kW][32]) const {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    Nb3<double>(*b)[32] = sh[z & 1];
    b[w][lane] = c;
    __syncthreads();  // buffer z&1 was last read two planes ago, before the previous barrier
    const Nb3<double> s = b[max(w - 1, 0)][lane], n = b[min(w + 1, kW - 1)][lane];
    Nb3<double> wv, e;
    wv.gcr = __shfl_up_sync(0xffffffffu, c.gcr, 1);
    wv.gnb = __shfl_up_sync(0xffffffffu, c.gnb, 1);
    wv.pd = __shfl_up_sync(0xffffffffu, c.pd, 1);
    wv.pl = __shfl_up_sync(0xffffffffu, c.pl, 1);
    e.gcr = __shfl_down_sync(0xffffffffu, c.gcr, 1);
    e.gnb = __shfl_down_sync(0xffffffffu, c.gnb, 1);
    e.pd = __shfl_down_sync(0xffffffffu, c.pd, 1);
    e.pl = __shfl_down_sync(0xffffffffu, c.pl, 1);
    if (!out) return;
    const ModelConst& M = a.m;
    // 7-point mask in the order z-1, y-1, x-1, centre, x+1, y+1, z+1
    const double mx = M.idx2[0], my = M.idx2[1], mz = M.idx2[2], mc = -2. * (mx + my + mz);
    auto lap = [&](double z0, double y0, double x0, double vc, double x1, double y1, double z1) {
      double v = mz * z0;
      v = fma(my, y0, v);
      v = fma(mx, x0, v);
      v = fma(mc, vc, v);
      v = fma(mx, x1, v);
      v = fma(my, y1, v);
      return fma(mz, z1, v);
    };
    const double lapCr = lap(up.gcr, s.gcr, wv.gcr, c.gcr, e.gcr, n.gcr, dn.gcr);
    const double lapNb = lap(up.gnb, s.gnb, wv.gnb, c.gnb, e.gnb, n.gnb, dn.gnb);
    const double lapD = lap(up.pd, s.pd, wv.pd, c.pd, e.pd, n.pd, dn.pd);
    const double lapL = lap(up.pl, s.pl, wv.pl, c.pl, e.pl, n.pl, dn.pl);
    const double X = rc.x, Y = rc.y, pd = c.pd, pl = c.pl;
    const double ocr = X + M.dt * (M.D[0][0] * lapCr + M.D[0][1] * lapNb);
    const double onb = Y + M.dt * (M.D[1][0] * lapCr + M.D[1][1] * lapNb);
    const double pD = p64(pd), pL = p64(pl), pG = 1.0 - pD - pL;
    Poly64 m;
    poly64(pD, pG, pL, m);
    const double gcr = c.gcr, gnb = c.gnb;
    const double gam = g64<0>(gcr, gnb);
    const double dgCr = dg64<0>(gcr, gnb), dgNb = dg64<1>(gcr, gnb);
    const double dCr = fict64<1, 0>(X, Y, m), dNb = fict64<1, 1>(X, Y, m);
    const double gpd = gam - g64<1>(dCr, dNb) - dgCr * (gcr - dCr) - dgNb * (gnb - dNb);
    const double dFd = -pp64(pd) * gpd + 2.0 * M.omega[0] * pd * (pd - 1.0) * (2.0 * pd - 1.0) +
                       2.0 * M.alpha * pd * pl * pl - M.kappa[0] * lapD;
    const double lCr = fict64<2, 0>(X, Y, m), lNb = fict64<2, 1>(X, Y, m);
    const double gpl = gam - g64<2>(lCr, lNb) - dgCr * (gcr - lCr) - dgNb * (gnb - lNb);
    const double dFl = -pp64(pl) * gpl + 2.0 * M.omega[1] * pl * (pl - 1.0) * (2.0 * pl - 1.0) +
                       2.0 * M.alpha * pl * pd * pd - M.kappa[1] * lapL;
    store64(static_cast<double*>(a.out[0]), a, cx, cy, z, ocr);
    store64(static_cast<double*>(a.out[1]), a, cx, cy, z, onb);
    store64(static_cast<double*>(a.out[2]), a, cx, cy, z, pd - M.dt * M.L[0] * dFd);
    store64(static_cast<double*>(a.out[3]), a, cx, cy, z, pl - M.dt * M.L[1] * dFl);
  }
};

__global__ void __launch_bounds__(32 * kW) k_stream3d_f64(Step3DArgs a) {
  __shared__ Nb3<double> sh[2][kW][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int x = blockIdx.x * kCols - 1 + lane;
  const int y = blockIdx.y * kRowsOut - 1 + w;
  const int z0 = blockIdx.z * a.zrows;
  const int z1 = min(z0 + a.zrows, a.Nz);
  const S64 S{a, min(max(x, 0), a.Nx - 1), min(max(y, 0), a.Ny - 1),
              lane >= 1 && lane <= kCols && w >= 1 && w <= kRowsOut && x < a.Nx && y < a.Ny};
  Raw3<double> r0 = S.load(z0), r1 = S.load(z0 + 1), r2;
  Nb3<double> n0 = S.solve(S.load(z0 - 1)), n1 = S.solve(r0), n2;
  int z = z0;
  for (; z + 2 < z1; z += 3) {
    r2 = S.load(z + 2);
    n2 = S.solve(r1);
    S.update(z, n0, n1, n2, r0, sh);
    r0 = S.load(z + 3);
    n0 = S.solve(r2);
    S.update(z + 1, n1, n2, n0, r1, sh);
    r1 = S.load(z + 4);
    n1 = S.solve(r0);
    S.update(z + 2, n2, n0, n1, r2, sh);
  }
  for (; z < z1; z++) {
    r2 = S.load(z + 2);
    n2 = S.solve(r1);
    S.update(z, n0, n1, n2, r0, sh);
    n0 = n1;
    n1 = n2;
    r0 = r1;
    r1 = r2;
  }
}

// ---- FP32 form, two planes per barrier ----
// A CTA covers 32 x-columns by 13 y-rows of output and streams along z.
// Warps 0..12 own one row each, every lane an output column; warps 13..15
// solve the 94 halo cells around the tile (the rows above and below, 34
// cells each, and the columns left and right, 13 cells each).  Every thread
// publishes its solved cell into a 15 x 34 plane in shared memory, and the
// row warps read all four in-plane neighbours from there (no shuffles); z
// neighbours come from a register window.  With 32 output columns per CTA a
// power-of-two grid side splits into whole tiles.
// Planes reach shared memory through a four-plane ring filled by TMA: one
// thread issues, per plane, a tiled copy of the CTA's 15 x 36 box of A
// records and one of B records, from two columns left of the tile (so that
// the box of 8-byte B records starts on a 16-byte boundary), both
// completing on the plane slot's mbarrier; every thread reads its own
// (clamped) record from the slot, at the same index in both boxes.  Records
// outside the grid arrive as zeros and are never read (threads past an edge
// read the clamped record).  Each
// iteration solves planes z+1 and z+2, publishes them and passes one barrier
// for both updates; a plane's record is read from the ring once, for its
// solve, and kept in registers until its update.
constexpr int kRing3 = 4;                      // planes in the ring (a power of two)
constexpr int kW3 = 16;                        // warps per CTA
constexpr int kRows3 = 13;                     // output rows (warps 0..12)
constexpr int kCols3 = 32;                     // output columns
constexpr int kPR = kRows3 + 2;                // rows of a staged or published plane
constexpr int kPC = kCols3 + 2;                // columns of a published plane
constexpr int kBox3 = kCols3 + 4;              // records per staged row, from x0 - 2
constexpr int kHalo3 = 2 * kPC + 2 * kRows3;   // halo cells (94 <= 3 warps)
static_assert(kHalo3 <= 32 * (kW3 - kRows3), "the halo warps cover the halo");
constexpr uint32_t kBoxBytesA = kPR * kBox3 * sizeof(float4);  // 8640
constexpr uint32_t kBoxBytesB = kPR * kBox3 * sizeof(uint2);   // 4320
constexpr uint32_t kSlotA = (kBoxBytesA + 127) / 128 * 128, kSlotB = (kBoxBytesB + 127) / 128 * 128;
constexpr uint32_t kTxPlane = kBoxBytesA + kBoxBytesB;  // bytes one plane's two copies deliver
struct Smem3 {
  float4 ra[kRing3][kSlotA / sizeof(float4)];
  uint2 rc[kRing3][kSlotB / sizeof(uint2)];
  // two published planes per iteration, two iterations; the cell past the
  // plane takes the writes of the two idle halo lanes
  Nb3<float> sh[4][kPR * kPC + 1];
  unsigned long long bar[kRing3];
};
static_assert(offsetof(Smem3, rc) % 128 == 0, "ring slots must stay 128-byte aligned");
constexpr size_t kSmem3 = sizeof(Smem3) + 128;  // + slack to align the base to 128 B

// gamma solve of one cell (warp-uniform bulk / equilibrium-referenced forms)
__device__ __forceinline__ Nb3<float> solve32(const Step3DArgs& a, const Raw3<float>& r) {
  const float2 h = cq_halves(r.cq.x);
  const float cx = h.x * kCqXi, cy = h.y * kCqXi;
  Nb3<float> n;
  n.pd = r.pd;
  n.pl = r.pl;
  if (__all_sync(0xffffffffu, fmaxf(fabsf(r.pd), fabsf(r.pl)) < kBulkPhi))
    gamma_bulk32(a.k, r.x, r.y, cx, cy, n.gcr, n.gnb);
  else
    gamma_u32(a.k, r.x, r.y, cx, cy, r.pd, r.pl, n.gcr, n.gnb);
  return n;
}

// update of one output cell (record i) from its seven neighbours' solves
__device__ __forceinline__ void update32(const Step3DArgs& a, long long i, const Nb3<float>& up,
                                         const Nb3<float>& c, const Nb3<float>& dn,
                                         const Nb3<float>& s, const Nb3<float>& n,
                                         const Nb3<float>& wv, const Nb3<float>& e,
                                         const Raw3<float>& rc) {
  const float i2x = a.idx2f[0], i2y = a.idx2f[1], i2z = a.idx2f[2];
  auto lap = [&](float z0, float y0, float x0, float vc, float x1, float y1, float z1) {
    const float sx = (x0 - vc) + (x1 - vc);
    const float sy = (y0 - vc) + (y1 - vc);
    const float sz = (z0 - vc) + (z1 - vc);
    return fmaf(sx, i2x, fmaf(sy, i2y, sz * i2z));
  };
  const float lapCr = lap(up.gcr, s.gcr, wv.gcr, c.gcr, e.gcr, n.gcr, dn.gcr);
  const float lapNb = lap(up.gnb, s.gnb, wv.gnb, c.gnb, e.gnb, n.gnb, dn.gnb);
  const float lapD = lap(up.pd, s.pd, wv.pd, c.pd, e.pd, n.pd, dn.pd);
  const float lapL = lap(up.pl, s.pl, wv.pl, c.pl, e.pl, n.pl, dn.pl);
  const float4 cc = cq_unpack(rc.cq);
  const float X = rc.x, Y = rc.y, pd = rc.pd, pl = rc.pl;
  const float ycr = fmaf(a.dtD[0][0], lapCr, a.dtD[0][1] * lapNb) - cc.x, tcr = X + ycr;
  const float ynb = fmaf(a.dtD[1][0], lapCr, a.dtD[1][1] * lapNb) - cc.y, tnb = Y + ynb;
  const FastCoef& K = a.k;
  const float u1 = c.gcr, u2 = c.gnb;
  const float dFd = fmaf(-a.kap[0], lapD, dF_local32(pd, pl, quad2(K.dP[0], u1, u2), a.om2[0], a.alpha2));
  const float dFl = fmaf(-a.kap[1], lapL, dF_local32(pl, pd, quad2(K.dP[1], u1, u2), a.om2[1], a.alpha2));
  const float yd = fmaf(-a.dtL[0], dFd, -cc.z), td = pd + yd;
  const float yl = fmaf(-a.dtL[1], dFl, -cc.w), tl = pl + yl;
  static_cast<float4*>(a.out[0])[i] = make_float4(tcr, tnb, td, tl);
  static_cast<uint2*>(a.out[1])[i] =
      cq_pack((tcr - X) - ycr, (tnb - Y) - ynb, (td - pd) - yd, (tl - pl) - yl);
}

// SKIP: the instantiation with the test hook (Step3DArgs::skip_plane)
template <bool SKIP>
__global__ void __launch_bounds__(32 * kW3, 2)
    k_stream3d_f32(Step3DArgs a, const __grid_constant__ Tma3 t) {
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = tma::smem_addr(smem_raw);
  Smem3& sm = *reinterpret_cast<Smem3*>(smem_raw + ((128u - (raw & 127u)) & 127u));
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int xa = blockIdx.x * kCols3 - 1;    // first column of the published plane
  const int yb = blockIdx.y * kRows3 - 1;    // first row of the staged boxes / published plane
  // this thread's cell in the published plane (pr, pc): a row warp's own
  // cell, or a halo cell (h = 94, 95 solve a duplicate and publish it past
  // the plane)
  const bool row = w < kRows3;
  int pr = w + 1, pc = lane + 1;
  bool pub = true;
  if (!row) {
    const int h = (w - kRows3) * 32 + lane;
    if (h < kPC) {
      pr = 0;
      pc = h;
    } else if (h < 2 * kPC) {
      pr = kPR - 1;
      pc = h - kPC;
    } else if (h < 2 * kPC + kRows3) {
      pr = 1 + h - 2 * kPC;
      pc = 0;
    } else {
      pr = 1 + min(h - 2 * kPC - kRows3, kRows3 - 1);
      pc = kPC - 1;
      pub = h < kHalo3;
    }
  }
  const int x = xa + pc, y = yb + pr;
  const int cx = min(max(x, 0), a.Nx - 1), cy = min(max(y, 0), a.Ny - 1);
  const bool out = row && x < a.Nx && y < a.Ny;
  // records in a plane and this thread's record in it: both below 2^31 (a
  // plane of records fits a 32-bit index; the plane offset is 64-bit)
  const int col = cy * a.pitch + cx, plane = a.Ny * a.pitch;
  const int ib = (cy - yb) * kBox3 + (cx - xa + 1);  // this thread's record in the staged boxes
  const int op = pub ? pr * kPC + pc : kPR * kPC;   // its cell in a published plane
  const int z0 = blockIdx.z * a.zrows;
  const int z1 = min(z0 + a.zrows, a.Nz);
  const uint32_t bar0 = tma::smem_addr(&sm.bar[0]);
  const uint32_t dA = tma::smem_addr(&sm.ra[0][0]), dB = tma::smem_addr(&sm.rc[0][0]);
  if (tid == 0) {
    tma::prefetch_map(&t.a);
    tma::prefetch_map(&t.b);
    for (int k = 0; k < kRing3; k++) tma::bar_init(bar0 + 8 * k, 1);
    tma::bar_init_fence();
  }
  __syncthreads();
  // plane p lives in ring slot (p - z0 + 1) & 3 and completes that slot's
  // phase (p - z0 + 1) >> 2; planes past z1 are never issued.  The slot
  // arguments below are compile-time constants.
  int last[kRing3] = {-2, -2, -2, -2};  // thread 0: last plane issued into each slot
  // A thread whose wait gave up stops waiting (later waits give up after
  // their first polls; it computes from whatever the ring holds and the
  // handle reports the failure); thread 0, once its own wait gave up, issues
  // nothing more, so the copies in flight are exactly those its final drain
  // waits for.  SKIP: the test hook that withholds one plane's copies in
  // the first CTA.
  bool gave_up = false;
  const bool skip =
      SKIP && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && a.skip_plane >= 0;
  auto issue = [&](int p, int sl) {
    if (tid == 0 && p <= z1 && !gave_up && !(skip && p == a.skip_plane)) {
      const int zc = min(max(p, 0), a.Nz - 1);
      tma::proxy_fence();  // the slot's earlier reads (ordered by the barrier) come first
      tma::bar_arrive_tx(bar0 + 8 * sl, kTxPlane);
      tma::load3(dA + sl * kSlotA, &t.a, 4 * (xa - 1), yb, zc, bar0 + 8 * sl);
      tma::load3(dB + sl * kSlotB, &t.b, 2 * (xa - 1), yb, zc, bar0 + 8 * sl);
      last[sl] = p;
    }
  };
  auto wait = [&](int p, int sl) {
    if (!tma::bar_wait(bar0 + 8 * sl, uint32_t((p - z0 + 1) >> 2) & 1u,
                       gave_up ? 0ull : tma::kWaitNs))
      gave_up = true;
  };
  auto fetch = [&](int sl) {
    const float4 v = sm.ra[sl][ib];
    return Raw3<float>{v.x, v.y, v.z, v.w, sm.rc[sl][ib]};
  };
  auto update = [&](int z, const Nb3<float>& up, const Nb3<float>& c, const Nb3<float>& dn,
                    const Raw3<float>& rc, const Nb3<float>* P) {
    if (out)
      update32(a, (long long)z * plane + col, up, c, dn, P[op - kPC], P[op + kPC], P[op - 1],
               P[op + 1], rc);
  };
  for (int k = -1; k <= 2; k++) issue(z0 + k, k + 1);
  wait(z0 - 1, 0);
  wait(z0, 1);
  Raw3<float> rB = fetch(1), rC, rD;  // raw records kept for the updates
  Nb3<float> nA = solve32(a, fetch(0)), nB = solve32(a, rB), nC, nD;
  __syncthreads();  // slots 0 and 1 are read before the first pair refills them
  // two planes z, z+1; issued up to plane z+2 on entry.  Q = (z - z0) & 3
  // (0 or 2) fixes the ring slots and the exchange slots.
  auto pair = [&](auto q, int z) {
    constexpr int Q = decltype(q)::value;
    constexpr int s1 = (2 + Q) & 3, s2 = (3 + Q) & 3, s3 = Q & 3, s4 = (1 + Q) & 3;
    // the slots of planes z-1 and z: read before the previous barrier
    issue(z + 3, s3);
    issue(z + 4, s4);
    wait(z + 1, s1);
    rC = fetch(s1);
    wait(z + 2, s2);
    rD = fetch(s2);
    nC = solve32(a, rC);
    nD = solve32(a, rD);
    Nb3<float>* b0 = sm.sh[Q];
    Nb3<float>* b1 = sm.sh[Q + 1];
    b0[op] = nB;
    b1[op] = nC;
    // these exchange slots were last read two pairs ago, before the previous
    // pair's barrier
    __syncthreads();
    update(z, nA, nB, nC, rB, b0);
    update(z + 1, nB, nC, nD, rC, b1);
    nA = nC;
    nB = nD;
    rB = rD;
  };
  int z = z0;
  for (; z + 3 < z1; z += 4) {
    pair(std::integral_constant<int, 0>{}, z);
    pair(std::integral_constant<int, 2>{}, z + 2);
  }
  int q = 0;  // (z - z0) & 3
  if (z + 1 < z1) {
    pair(std::integral_constant<int, 0>{}, z);
    z += 2;
    q = 2;
  }
  if (z < z1) {  // one plane left; plane z+1 (<= z1) was issued by the last pair
    const int s1 = (2 + q) & 3;
    wait(z + 1, s1);
    nC = solve32(a, fetch(s1));
    Nb3<float>* b0 = sm.sh[q];
    b0[op] = nB;
    __syncthreads();
    update(z, nA, nB, nC, rB, b0);
  }
  if (gave_up && a.status) atomicExch(a.status, 3);
  // thread 0 waits for every plane it issued, so its copies have all landed
  // unless one of its waits gave up: then it waits again (bounded) before
  // the block exits
  if (tid == 0 && gave_up)
    for (int k = 0; k < kRing3; k++)
      if (last[k] >= z0 - 1) tma::bar_wait(bar0 + 8 * k, uint32_t((last[k] - z0 + 1) >> 2) & 1u);
}

// FP64 ghost-ring fields <-> FP32 records (3D): a thread per cell, the
// launch grid covering (x, y) with its blocks and z with gridDim.z (looping
// when Nz exceeds it), so no index needs a division
__global__ void k_import3d(Conv3DArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.Nx || y >= a.Ny) return;
  for (int z = blockIdx.z; z < a.Nz; z += gridDim.z) {
    const long long i64 = ((long long)(z + 1) * (a.Ny + 2) + (y + 1)) * (a.Nx + 2) + (x + 1);
    const long long r = ((long long)z * a.Ny + y) * a.pitch32 + x;
    float hi[4], c[4];
#pragma unroll
    for (int k = 0; k < 4; k++) split_f64(a.f64[k][i64], hi[k], c[k]);  // value = hi - c
    reinterpret_cast<float4*>(a.A)[r] = make_float4(hi[0], hi[1], hi[2], hi[3]);
    static_cast<uint2*>(a.B)[r] = cq_pack(c[0], c[1], c[2], c[3]);
  }
}

__global__ void k_export3d(Conv3DArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.Nx || y >= a.Ny) return;
  Step3DArgs g{};
  g.Nx = a.Nx;
  g.Ny = a.Ny;
  g.Nz = a.Nz;
  g.pitch = a.Nx + 2;
  for (int z = blockIdx.z; z < a.Nz; z += gridDim.z) {
    const long long r = ((long long)z * a.Ny + y) * a.pitch32 + x;
    const float4 v = reinterpret_cast<const float4*>(a.A)[r];
    const float4 c = cq_unpack(static_cast<const uint2*>(a.B)[r]);
    store64(a.f64[0], g, x, y, z, double(v.x) - double(c.x));
    store64(a.f64[1], g, x, y, z, double(v.y) - double(c.y));
    store64(a.f64[2], g, x, y, z, double(v.z) - double(c.z));
    store64(a.f64[3], g, x, y, z, double(v.w) - double(c.w));
  }
}

// z planes per segment: fill whole waves of resident CTAs, two extra planes
// of gamma solves per segment; tiles of tx x ty output cells per plane
int segment_planes(int Nx, int Ny, int Nz, int resident, int tx, int ty) {
  const long long cols = (long long)((Nx + tx - 1) / tx) * ((Ny + ty - 1) / ty);
  int best = Nz;
  double best_score = 0.0;
  for (int waves = 1; waves <= 256; waves++) {
    const long long segs = (long long)waves * resident / cols;
    if (segs < 1) continue;
    const int planes = int((Nz + segs - 1) / segs);
    if (planes < 16 && segs > 1) break;
    const long long used = cols * ((Nz + planes - 1) / planes);
    const long long slots = ((used + resident - 1) / resident) * (long long)resident;
    const double score = double(used) / double(slots) / (1.0 + 2.0 / planes);
    if (score > best_score) {
      best_score = score;
      best = planes;
    }
  }
  return best;
}

int g_resident3[2] = {0, 0};

template <bool F64>
cudaError_t query3() {
  int dev = 0, sms = 0, per = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) {
    if (F64)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_stream3d_f64, 32 * kW, 0);
    else
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_stream3d_f32<false>, 32 * kW3, kSmem3);
  }
  g_resident3[F64] = sms * (per > 0 ? per : 1);
  return e;
}

}  // namespace

cudaError_t prepare_step3d() {
  cudaError_t e = cudaFuncSetAttribute(k_stream3d_f32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(kSmem3));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_stream3d_f32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(kSmem3));
  if (e == cudaSuccess) e = query3<true>();
  return e == cudaSuccess ? query3<false>() : e;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library links the static runtime, not the driver library)
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                 const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                 const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

cudaError_t encode_step3d_maps(Tma3* t, const void* A, const void* B, int Nx, int Ny, int Nz,
                               int pitch) {
  static EncodeTiled encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    const cudaError_t e =
        cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    encode = reinterpret_cast<EncodeTiled>(fn);
  }
  const cuuint32_t box_a[3] = {4 * kBox3, kPR, 1}, box_b[3] = {2 * kBox3, kPR, 1}, one[3] = {1, 1, 1};
  const cuuint64_t dim_a[3] = {4ull * Nx, cuuint64_t(Ny), cuuint64_t(Nz)};
  const cuuint64_t dim_b[3] = {2ull * Nx, cuuint64_t(Ny), cuuint64_t(Nz)};
  const cuuint64_t str_a[2] = {16ull * pitch, 16ull * pitch * Ny};
  const cuuint64_t str_b[2] = {8ull * pitch, 8ull * pitch * Ny};
  CUresult r = encode(&t->a, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(A), dim_a, str_a,
                      box_a, one, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r == CUDA_SUCCESS)
    r = encode(&t->b, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<void*>(B), dim_b, str_b, box_b,
               one, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_step3d(Step3DArgs a, bool f64, const Tma3* t, cudaStream_t s) {
  const int resident = g_resident3[f64] > 0 ? g_resident3[f64] : 152;
  const int tx = f64 ? kCols : kCols3, ty = f64 ? kRowsOut : kRows3;
  a.zrows = segment_planes(a.Nx, a.Ny, a.Nz, resident, tx, ty);
  dim3 grid((a.Nx + tx - 1) / tx, (a.Ny + ty - 1) / ty, (a.Nz + a.zrows - 1) / a.zrows);
  if (f64) {
    k_stream3d_f64<<<grid, 32 * kW, 0, s>>>(a);
  } else {
    if (!t) return cudaErrorInvalidValue;
    if (a.skip_plane >= 0)
      k_stream3d_f32<true><<<grid, 32 * kW3, kSmem3, s>>>(a, *t);
    else
      k_stream3d_f32<false><<<grid, 32 * kW3, kSmem3, s>>>(a, *t);
  }
  return cudaGetLastError();
}

dim3 conv3d_grid(const Conv3DArgs& a) {
  return dim3((a.Nx + 31) / 32, (a.Ny + 7) / 8, std::min(a.Nz, 65535));
}

cudaError_t launch_import3d(const Conv3DArgs& a, cudaStream_t s) {
  k_import3d<<<conv3d_grid(a), dim3(32, 8), 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_export3d(const Conv3DArgs& a, cudaStream_t s) {
  k_export3d<<<conv3d_grid(a), dim3(32, 8), 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pfa
