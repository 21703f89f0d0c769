// pfa_step2d_f32.cu -- the FP32 precision form of the 2D step (sm_103a).
//
// Same step as the FP64 kernel (src/main.cpp:289-305 fused), arithmetic in
// FP32, x_Cr / x_Nb Kahan-compensated, phases in 32-bit fixed point (or FP32
// + Kahan).  Organised for instruction economy, since at 48 bytes per cell
// the HBM budget leaves ~200 FP32 instructions per cell:
//  * each warp owns a strip of 32 columns and streams down H rows; the three
//    rows a 5-point Laplacian needs live in registers (a sliding window), so
//    every cell's gamma solve runs once and nothing goes through shared
//    memory;
//  * left / right neighbours come from __shfl_up / __shfl_down; the two
//    columns outside the strip are computed by lanes 0 and 31 in one
//    divergent pass per row;
//  * the raw fields of the row after next are loaded one iteration ahead.
//
// Compact layout: Ny rows of `pitch` elements (pitch a multiple of 32, rows
// 128-byte aligned), interior cell (x, y) at y * pitch + x, no ghost ring;
// zero-flux edges come from clamped indexing (the mirror the reference's
// halo fill produces).
#include <cstdint>
#include <type_traits>

#include "pfa_device.cuh"
#include "pfa_kernels.h"

namespace pfa {

using namespace dev;

namespace {

constexpr int kWarps = 4;         // warps (strips) per CTA
constexpr int kCols = 30;         // output columns per warp; lanes 0 and 31 are halo

// The values a neighbour needs: gamma compositions and the phases (FP32).
struct Nb {
  float gcr, gnb, pd, pl;
};

template <bool FIX>
using PhiT = typename std::conditional<FIX, int, float>::type;

// Raw stored values of one cell.
template <bool FIX>
struct Raw {
  float x, y;
  PhiT<FIX> pd, pl;
};

template <bool FIX>
__device__ __forceinline__ float phf(PhiT<FIX> v) {
  if constexpr (FIX)
    return phi_of(v);
  else
    return v;
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
  const float t = fmaf(-ph, ph, ph);                 // phi (1 - phi)
  const float pp = 30.0f * t * t;                    // p'(phi)
  const float well = ph * fmaf(ph, fmaf(2.0f * om2, ph, -3.0f * om2), om2);
  return fmaf(-pp, dP, fmaf(alpha2 * ph, pj * pj, well));
}

template <bool FIX>
struct Stream {
  const Step2DArgs& a;
  const float *px, *py, *pc0, *pc1, *pc2, *pc3;
  const PhiT<FIX>*pd, *pl;
  float *ox, *oy, *oc0, *oc1, *oc2, *oc3;
  PhiT<FIX>*od, *ol;
  int Ny, P;
  bool out;  // this lane writes its column

  __device__ __forceinline__ int row(int y) const { return min(max(y, 0), Ny - 1) * P; }

  __device__ __forceinline__ Raw<FIX> load(int off) const {
    return Raw<FIX>{__ldg(px + off), __ldg(py + off), __ldg(pd + off), __ldg(pl + off)};
  }

  // update row y from its window (up, c, dn); rc = raw centre values
  __device__ __forceinline__ void update(int y, const Nb& up, const Nb& c, const Nb& dn,
                                         const Raw<FIX>& rc) const {
    const int i = y * P;
    const float cin0 = __ldg(pc0 + i), cin1 = __ldg(pc1 + i);
    float cin2 = 0.f, cin3 = 0.f;
    if constexpr (!FIX) {
      cin2 = __ldg(pc2 + i);
      cin3 = __ldg(pc3 + i);
    }
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
    const float X = rc.x, Y = rc.y;
    const float ycr = fmaf(a.dtD[0][0], lapCr, a.dtD[0][1] * lapNb) - cin0, tcr = X + ycr;
    const float ynb = fmaf(a.dtD[1][0], lapCr, a.dtD[1][1] * lapNb) - cin1, tnb = Y + ynb;
    // Allen-Cahn
    const FastCoef& K = a.k;
    const float u1 = c.gcr - K.xe_gam[0], u2 = c.gnb - K.xe_gam[1];
    const float dFd = fmaf(-a.kap[0], lapD, dF_local(c.pd, c.pl, quad2(K.dP[0], u1, u2), a.om2[0], a.alpha2));
    const float dFl = fmaf(-a.kap[1], lapL, dF_local(c.pl, c.pd, quad2(K.dP[1], u1, u2), a.om2[1], a.alpha2));
    if (out) {
      ox[i] = tcr;
      oy[i] = tnb;
      oc0[i] = (tcr - X) - ycr;
      oc1[i] = (tnb - Y) - ynb;
      if constexpr (FIX) {
        od[i] = phi_step(rc.pd, -a.dtL[0] * dFd);
        ol[i] = phi_step(rc.pl, -a.dtL[1] * dFl);
      } else {
        const float yd = fmaf(-a.dtL[0], dFd, -cin2), td = c.pd + yd;
        const float yl = fmaf(-a.dtL[1], dFl, -cin3), tl = c.pl + yl;
        od[i] = td;
        ol[i] = tl;
        oc2[i] = (td - c.pd) - yd;
        oc3[i] = (tl - c.pl) - yl;
      }
    }
  }
};

template <bool FIX>
__global__ void __launch_bounds__(32 * kWarps, 8) k_stream_f32(Step2DArgs a) {
  const int lane = threadIdx.x & 31;
  const int strip = blockIdx.x * kWarps + (threadIdx.x >> 5);
  const int x0 = strip * kCols;  // first output column of the strip
  if (x0 >= a.Nx) return;        // whole warp leaves together
  const int y0 = blockIdx.y * a.rows;
  const int y1 = min(y0 + a.rows, a.Ny);
  const int gx = x0 - 1 + lane;  // lanes 0 and 31 hold the neighbour columns
  const int cx = min(max(gx, 0), a.Nx - 1);
  const FastCoef& K = a.k;
  Stream<FIX> S{a,
                static_cast<const float*>(a.in[0]) + cx, static_cast<const float*>(a.in[1]) + cx,
                a.cin[0] + cx, a.cin[1] + cx, FIX ? nullptr : a.cin[2] + cx,
                FIX ? nullptr : a.cin[3] + cx,
                static_cast<const PhiT<FIX>*>(a.in[2]) + cx, static_cast<const PhiT<FIX>*>(a.in[3]) + cx,
                static_cast<float*>(a.out[0]) + cx, static_cast<float*>(a.out[1]) + cx,
                a.cout[0] + cx, a.cout[1] + cx, FIX ? nullptr : a.cout[2] + cx,
                FIX ? nullptr : a.cout[3] + cx,
                static_cast<PhiT<FIX>*>(a.out[2]) + cx, static_cast<PhiT<FIX>*>(a.out[3]) + cx,
                a.Ny, a.pitch, lane >= 1 && lane <= kCols && gx < a.Nx};
  auto solve_raw = [&](const Raw<FIX>& r) {
    return solve(K, r.x, r.y, phf<FIX>(r.pd), phf<FIX>(r.pl));
  };
  // window rows y-1, y, y+1 and raw rows y, y+1, y+2
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

// ---- layout conversion between the reference's FP64 fields and the form ----
__global__ void k_import_compact(ConvArgs a) {
  const int gx = blockIdx.x * blockDim.x + threadIdx.x;
  const int gy = blockIdx.y * blockDim.y + threadIdx.y;
  if (gx >= a.Nx || gy >= a.Ny) return;
  const size_t i64 = size_t(gy + 1) * a.pitch64 + gx + 1;
  const size_t i32 = size_t(gy) * a.pitch32 + gx;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const double v = a.f64[k][i64];
    if (k >= 2 && a.phi_fix) {
      reinterpret_cast<int*>(a.f32[k])[i32] = phi_quantize(v);
      continue;
    }
    const float hi = float(v);
    a.f32[k][i32] = hi;
    // compensation c holds -(low part): value = hi - c
    if (a.c32[k]) a.c32[k][i32] = float(double(hi) - v);
  }
}

__global__ void k_export_compact(ConvArgs a) {
  const int gx = blockIdx.x * blockDim.x + threadIdx.x;
  const int gy = blockIdx.y * blockDim.y + threadIdx.y;
  if (gx >= a.Nx || gy >= a.Ny) return;
  const size_t i32 = size_t(gy) * a.pitch32 + gx;
  const size_t row = size_t(gy + 1) * a.pitch64;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    double v;
    if (k >= 2 && a.phi_fix) {
      v = double(reinterpret_cast<const int*>(a.f32[k])[i32]) * kPhiInvScaleD;
    } else {
      v = double(a.f32[k][i32]);
      if (a.c32[k]) v -= double(a.c32[k][i32]);
    }
    double* f = a.f64[k];
    f[row + gx + 1] = v;
    // ghost ring = mirror of the interior; corners take the diagonal cell
    const bool l = gx == 0, r = gx == a.Nx - 1, b = gy == 0, t = gy == a.Ny - 1;
    if (l) f[row] = v;
    if (r) f[row + a.Nx + 1] = v;
    if (b) {
      f[gx + 1] = v;
      if (l) f[0] = v;
      if (r) f[a.Nx + 1] = v;
    }
    if (t) {
      const size_t top = size_t(a.Ny + 1) * a.pitch64;
      f[top + gx + 1] = v;
      if (l) f[top] = v;
      if (r) f[top + a.Nx + 1] = v;
    }
  }
}

// Rows per warp segment: the CTA count should fill whole waves of the
// resident CTAs (a partial last wave idles SMs), while each segment pays two
// extra rows of gamma solves at its ends.
static int segment_rows(int Nx, int Ny, int resident) {
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

static int g_resident[2] = {0, 0};  // resident CTAs of the two variants

template <bool FIX>
static cudaError_t query_resident() {
  int dev = 0, sms = 0, per = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_stream_f32<FIX>, 32 * kWarps, 0);
  g_resident[FIX] = sms * (per > 0 ? per : 1);
  return e;
}

template <bool FIX>
static cudaError_t launch_stream(Step2DArgs a, cudaStream_t s) {
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
  cudaError_t e = query_resident<true>();
  return e == cudaSuccess ? query_resident<false>() : e;
}

cudaError_t launch_import_f32(const ConvArgs& a, cudaStream_t s) {
  dim3 block(32, 8);
  dim3 grid((a.Nx + 31) / 32, (a.Ny + 7) / 8);
  k_import_compact<<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_export_f32(const ConvArgs& a, cudaStream_t s) {
  dim3 block(32, 8);
  dim3 grid((a.Nx + 31) / 32, (a.Ny + 7) / 8);
  k_export_compact<<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pfa
