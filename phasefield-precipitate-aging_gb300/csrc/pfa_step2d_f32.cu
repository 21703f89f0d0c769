// pfa_step2d_f32.cu -- the FP32 precision form of the 2D step (sm_103a).
//
// Same step as the FP64 kernel (src/main.cpp:289-305 fused), arithmetic in
// FP32, x_Cr / x_Nb Kahan-compensated, phases in 32-bit fixed point (or FP32
// + Kahan).  At 48 bytes per cell the HBM budget leaves ~250 instructions per
// cell, so the kernel is organised for instruction economy:
//  * each warp owns a strip of 30 output columns (lanes 1..30; lanes 0 and
//    31 carry the neighbour columns) and streams down a segment of rows; the
//    three rows a 5-point Laplacian needs live in registers, rotated by a
//    3x-unrolled loop, so each cell's gamma solve runs once and nothing goes
//    through shared memory;
//  * left / right neighbours come from __shfl_up / __shfl_down;
//  * the state is stored as two records per cell -- A = {x_Cr, x_Nb, phi_del,
//    phi_lav} (16 bytes) and B = Kahan compensations {c_Cr, c_Nb} (8 bytes,
//    or 16 with compensated phases) -- so a row costs one 128-bit and one
//    64-bit load and store and a single address per lane; records of the row
//    after next are loaded one iteration ahead.
//
// Record layout: Ny rows of `pitch` records (pitch a multiple of 32), interior
// cell (x, y) at record y * pitch + x, no ghost ring; zero-flux edges come
// from clamped indexing (the mirror the reference's halo fill produces).
// Fixed-point phases (FIX) keep their int32 bits in the float slots.
#include <cstdint>
#include <type_traits>

#include "pfa_device.cuh"
#include "pfa_kernels.h"

namespace pfa {

using namespace dev;

namespace {

constexpr int kWarps = 4;  // warps (strips) per CTA
constexpr int kCols = 30;  // output columns per warp; lanes 0 and 31 are halo

// The values a neighbour needs: gamma compositions and the phases (FP32).
struct Nb {
  float gcr, gnb, pd, pl;
};

// Compensation record: {c_Cr, c_Nb} or {c_Cr, c_Nb, c_del, c_lav}.
template <bool FIX>
using CompT = typename std::conditional<FIX, float2, float4>::type;

template <bool FIX>
struct Raw {
  float4 a;      // x_Cr, x_Nb, phi_del, phi_lav (int bits when FIX)
  CompT<FIX> c;  // Kahan compensations
};

template <bool FIX>
__device__ __forceinline__ float phf(float bits) {
  if constexpr (FIX)
    return phi_of(__float_as_int(bits));
  else
    return bits;
}

// gamma solve of one cell (approximate reciprocal: 2 ulp is far inside the
// form's error budget)
__device__ __forceinline__ Nb solve(const FastCoef& K, float X, float Y, float phd, float phl) {
  const float pD = p32(phd), pL = p32(phl);
  const float pG = p_gamma32(phd, phl, pD, pL);
  const float m0 = pD * pD, m1 = pD * pG, m2 = pD * pL, m3 = pG * pG, m4 = pG * pL, m5 = pL * pL;
  const float* d = K.den;
  const float den = fmaf(d[0], m0, fmaf(d[1], m1, fmaf(d[2], m2, fmaf(d[3], m3, fmaf(d[4], m4, d[5] * m5)))));
  const float r = __fdividef(1.0f, den);
  float n[2];
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const float* a = K.num[c];
    const float lx = fmaf(a[0], pD, fmaf(a[1], pG, a[2] * pL));
    const float ly = fmaf(a[3], pD, fmaf(a[4], pG, a[5] * pL));
    const float q = fmaf(a[6], m0, fmaf(a[7], m1, fmaf(a[8], m2, fmaf(a[9], m3, fmaf(a[10], m4, a[11] * m5)))));
    n[c] = fmaf(X, lx, fmaf(Y, ly, q));
  }
  return Nb{n[0] * r, n[1] * r, phd, phl};
}

__device__ __forceinline__ int add_sat(int a, int b) {
  int r;
  asm("add.sat.s32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}

// q + round(inc 2^29) with saturation; |q| stays <= kPhiQMax so that two
// values differ by less than 2^31
__device__ __forceinline__ int phi_step(int q, float inc) {
  const int d = __float2int_rn(inc * kPhiScale);  // saturates on overflow
  return max(-kPhiQMax, min(kPhiQMax, add_sat(q, d)));
}

// dF/dphi_i without the Laplacian term: -p'(phi) dP + 2 omega phi (phi-1)(2 phi-1)
// + 2 alpha phi phi_j^2, Horner forms
__device__ __forceinline__ float dF_local(float ph, float pj, float dP, float om2, float alpha2) {
  const float t = fmaf(-ph, ph, ph);  // phi (1 - phi)
  const float pp = 30.0f * t * t;     // p'(phi)
  const float well = ph * fmaf(ph, fmaf(2.0f * om2, ph, -3.0f * om2), om2);
  return fmaf(-pp, dP, fmaf(alpha2 * ph, pj * pj, well));
}

template <bool FIX>
struct Stream {
  const Step2DArgs& a;
  const float4* A;        // this lane's column, row 0
  const CompT<FIX>* B;
  float4* Ao;
  CompT<FIX>* Bo;
  int Ny, P;
  bool out;  // this lane writes its column

  __device__ __forceinline__ int row(int y) const { return min(max(y, 0), Ny - 1) * P; }

  __device__ __forceinline__ Raw<FIX> load(int off) const { return Raw<FIX>{__ldg(A + off), __ldg(B + off)}; }

  // update row y from its window (up, c, dn); rc = raw centre record
  __device__ __forceinline__ void update(int y, const Nb& up, const Nb& c, const Nb& dn,
                                         const Raw<FIX>& rc) const {
    Nb w, e;
    w.gcr = __shfl_up_sync(0xffffffffu, c.gcr, 1);
    w.gnb = __shfl_up_sync(0xffffffffu, c.gnb, 1);
    w.pd = __shfl_up_sync(0xffffffffu, c.pd, 1);
    w.pl = __shfl_up_sync(0xffffffffu, c.pl, 1);
    e.gcr = __shfl_down_sync(0xffffffffu, c.gcr, 1);
    e.gnb = __shfl_down_sync(0xffffffffu, c.gnb, 1);
    e.pd = __shfl_down_sync(0xffffffffu, c.pd, 1);
    e.pl = __shfl_down_sync(0xffffffffu, c.pl, 1);
    const float idx2 = a.idx2f[0], idy2 = a.idx2f[1];
    auto lap = [&](float vw, float ve, float vn, float vs, float vc) {
      const float sx = (vw - vc) + (ve - vc);
      const float sy = (vn - vc) + (vs - vc);
      return fmaf(sx, idx2, sy * idy2);
    };
    const float lapCr = lap(w.gcr, e.gcr, up.gcr, dn.gcr, c.gcr);
    const float lapNb = lap(w.gnb, e.gnb, up.gnb, dn.gnb, c.gnb);
    const float lapD = lap(w.pd, e.pd, up.pd, dn.pd, c.pd);
    const float lapL = lap(w.pl, e.pl, up.pl, dn.pl, c.pl);
    // Cahn-Hilliard, Kahan-compensated
    const float X = rc.a.x, Y = rc.a.y;
    const float ycr = fmaf(a.dtD[0][0], lapCr, a.dtD[0][1] * lapNb) - rc.c.x, tcr = X + ycr;
    const float ynb = fmaf(a.dtD[1][0], lapCr, a.dtD[1][1] * lapNb) - rc.c.y, tnb = Y + ynb;
    // Allen-Cahn
    const FastCoef& K = a.k;
    const float u1 = c.gcr - K.xe_gam[0], u2 = c.gnb - K.xe_gam[1];
    const float dFd = fmaf(-a.kap[0], lapD, dF_local(c.pd, c.pl, quad2(K.dP[0], u1, u2), a.om2[0], a.alpha2));
    const float dFl = fmaf(-a.kap[1], lapL, dF_local(c.pl, c.pd, quad2(K.dP[1], u1, u2), a.om2[1], a.alpha2));
    if (out) {
      const int i = y * P;
      float4 o;
      CompT<FIX> oc;
      o.x = tcr;
      o.y = tnb;
      oc.x = (tcr - X) - ycr;
      oc.y = (tnb - Y) - ynb;
      if constexpr (FIX) {
        o.z = __int_as_float(phi_step(__float_as_int(rc.a.z), -a.dtL[0] * dFd));
        o.w = __int_as_float(phi_step(__float_as_int(rc.a.w), -a.dtL[1] * dFl));
      } else {
        const float yd = fmaf(-a.dtL[0], dFd, -rc.c.z), td = c.pd + yd;
        const float yl = fmaf(-a.dtL[1], dFl, -rc.c.w), tl = c.pl + yl;
        o.z = td;
        o.w = tl;
        oc.z = (td - c.pd) - yd;
        oc.w = (tl - c.pl) - yl;
      }
      Ao[i] = o;
      Bo[i] = oc;
    }
  }
};

// One warp updates the strip of output columns x0 .. x0+29 over rows
// y0 .. y1-1 of one grid (the unit of work of both the single-grid and the
// batched kernels).  Whole warp; x0 < Nx.
template <bool FIX>
__device__ __forceinline__ void stream_strip(const Step2DArgs& a, const float4* Ain,
                                             const CompT<FIX>* Bin, float4* Aout,
                                             CompT<FIX>* Bout, int Nx, int Ny, int P, int x0,
                                             int y0, int y1) {
  const int lane = threadIdx.x & 31;
  const int gx = x0 - 1 + lane;  // lanes 0 and 31 hold the neighbour columns
  const int cx = min(max(gx, 0), Nx - 1);
  const FastCoef& K = a.k;
  const Stream<FIX> S{a, Ain + cx, Bin + cx, Aout + cx, Bout + cx,
                      Ny, P, lane >= 1 && lane <= kCols && gx < Nx};
  auto solve_raw = [&](const Raw<FIX>& r) {
    return solve(K, r.a.x, r.a.y, phf<FIX>(r.a.z), phf<FIX>(r.a.w));
  };
  // window rows y-1, y, y+1 and raw records of rows y, y+1, y+2
  Raw<FIX> r0 = S.load(S.row(y0)), r1 = S.load(S.row(y0 + 1)), r2;
  Nb n0 = solve_raw(S.load(S.row(y0 - 1))), n1 = solve_raw(r0), n2;
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
}

template <bool FIX>
__global__ void __launch_bounds__(32 * kWarps, 8) k_stream_f32(Step2DArgs a) {
  const int strip = blockIdx.x * kWarps + (threadIdx.x >> 5);
  const int x0 = strip * kCols;  // first output column of the strip
  if (x0 >= a.Nx) return;        // whole warp leaves together
  const int y0 = blockIdx.y * a.rows;
  stream_strip<FIX>(a, static_cast<const float4*>(a.in[0]),
                    static_cast<const CompT<FIX>*>(a.in[1]), static_cast<float4*>(a.out[0]),
                    static_cast<CompT<FIX>*>(a.out[1]), a.Nx, a.Ny, a.pitch, x0, y0,
                    min(y0 + a.rows, a.Ny));
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
__global__ void __launch_bounds__(32 * kWarps, 8) k_batch_f32(Step2DArgs a, BatchArgs b) {
  const int p = b.parity;
  if (blockIdx.x == 0 && threadIdx.x == 0) b.counter[p ^ 1] = 0;
  const int units = b.counter[2];
  for (;;) {
    int u = 0;
    if ((threadIdx.x & 31) == 0) u = atomicAdd(b.counter + p, 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= units) return;
    const BatchUnit w = b.unit[u];
    const BatchGrid& g = b.grid[w.grid];
    stream_strip<true>(a, g.A[p], g.B[p], g.A[p ^ 1], g.B[p ^ 1], g.Nx, g.Ny, g.pitch, w.x0,
                       w.y0, w.y1);
  }
}

// ---- layout conversion between the reference's FP64 fields and the form ----
__global__ void k_import_records(ConvArgs a) {
  const int gx = blockIdx.x * blockDim.x + threadIdx.x;
  const int gy = blockIdx.y * blockDim.y + threadIdx.y;
  if (gx >= a.Nx || gy >= a.Ny) return;
  const size_t i64 = size_t(gy + 1) * a.pitch64 + gx + 1;
  const size_t r = size_t(gy) * a.pitch32 + gx;
  float* A = a.A + 4 * r;
  float* B = a.B + size_t(a.bstride) * r;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const double v = a.f64[k][i64];
    if (k >= 2 && a.phi_fix) {
      A[k] = __int_as_float(phi_quantize(v));
      continue;
    }
    const float hi = float(v);
    A[k] = hi;
    // compensation c holds -(low part): value = hi - c
    if (k < a.bstride) B[k] = float(double(hi) - v);
  }
}

__global__ void k_export_records(ConvArgs a) {
  const int gx = blockIdx.x * blockDim.x + threadIdx.x;
  const int gy = blockIdx.y * blockDim.y + threadIdx.y;
  if (gx >= a.Nx || gy >= a.Ny) return;
  const size_t r = size_t(gy) * a.pitch32 + gx;
  const float* A = a.A + 4 * r;
  const float* B = a.B + size_t(a.bstride) * r;
  const size_t row = size_t(gy + 1) * a.pitch64;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    double v;
    if (k >= 2 && a.phi_fix) {
      v = double(__float_as_int(A[k])) * kPhiInvScaleD;
    } else {
      v = double(A[k]);
      if (k < a.bstride) v -= double(B[k]);
    }
    double* f = a.f64[k];
    f[row + gx + 1] = v;
    // ghost ring = mirror of the interior; corners take the diagonal cell
    const bool l = gx == 0, rr = gx == a.Nx - 1, b = gy == 0, t = gy == a.Ny - 1;
    if (l) f[row] = v;
    if (rr) f[row + a.Nx + 1] = v;
    if (b) {
      f[gx + 1] = v;
      if (l) f[0] = v;
      if (rr) f[a.Nx + 1] = v;
    }
    if (t) {
      const size_t top = size_t(a.Ny + 1) * a.pitch64;
      f[top + gx + 1] = v;
      if (l) f[top] = v;
      if (rr) f[top + a.Nx + 1] = v;
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

int g_resident[3] = {0, 0, 0};  // resident CTAs: the two variants, the batch kernel

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

template <bool FIX>
cudaError_t launch_stream(Step2DArgs a, cudaStream_t s) {
  const int resident = g_resident[FIX] > 0 ? g_resident[FIX] : 152 * 8;
  a.rows = segment_rows(a.Nx, a.Ny, resident);
  const int strips = (a.Nx + kCols - 1) / kCols;
  dim3 grid((strips + kWarps - 1) / kWarps, (a.Ny + a.rows - 1) / a.rows);
  k_stream_f32<FIX><<<grid, 32 * kWarps, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_step2d_f32(const Step2DArgs& a, cudaStream_t s) {
  return a.kahan_phi ? launch_stream<false>(a, s) : launch_stream<true>(a, s);
}

// occupancy of the FP32 kernels on the current device (outside any capture)
cudaError_t prepare_step2d_f32() {
  cudaError_t e = query_resident(k_stream_f32<false>, 0);
  if (e == cudaSuccess) e = query_resident(k_stream_f32<true>, 1);
  if (e == cudaSuccess) e = query_resident(k_batch_f32, 2);
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
  dim3 block(32, 8);
  dim3 grid((a.Nx + 31) / 32, (a.Ny + 7) / 8);
  k_import_records<<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_export_f32(const ConvArgs& a, cudaStream_t s) {
  dim3 block(32, 8);
  dim3 grid((a.Nx + 31) / 32, (a.Ny + 7) / 8);
  k_export_records<<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pfa
