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

constexpr int kRows = 64;         // rows per warp segment
constexpr int kWarps = 4;         // warps (strips) per CTA

// Per-cell values a neighbour needs: gamma compositions and the phases.
template <bool FIX>
struct Nb {
  float gcr, gnb;
  typename std::conditional<FIX, int, float>::type pd, pl;
};

// Raw stored values of one cell.
template <bool FIX>
struct Raw {
  float x, y;
  typename std::conditional<FIX, int, float>::type pd, pl;
};

template <bool FIX>
__device__ __forceinline__ Raw<FIX> load_raw(const Step2DArgs& a, size_t i) {
  Raw<FIX> r;
  r.x = __ldg(static_cast<const float*>(a.in[0]) + i);
  r.y = __ldg(static_cast<const float*>(a.in[1]) + i);
  if (FIX) {
    r.pd = __ldg(static_cast<const int*>(a.in[2]) + i);
    r.pl = __ldg(static_cast<const int*>(a.in[3]) + i);
  } else {
    r.pd = __ldg(static_cast<const float*>(a.in[2]) + i);
    r.pl = __ldg(static_cast<const float*>(a.in[3]) + i);
  }
  return r;
}

template <bool FIX>
__device__ __forceinline__ float phf(typename std::conditional<FIX, int, float>::type v) {
  if constexpr (FIX)
    return phi_of(v);
  else
    return v;
}

// gamma solve of one cell
template <bool FIX>
__device__ __forceinline__ Nb<FIX> solve(const FastCoef& K, const Raw<FIX>& r) {
  const float phd = phf<FIX>(r.pd), phl = phf<FIX>(r.pl);
  const float pD = p32(phd), pL = p32(phl);
  Nb<FIX> n;
  fict_gam32(K, r.x, r.y, pD, p_gamma32(phd, phl, pD, pL), pL, n.gcr, n.gnb);
  n.pd = r.pd;
  n.pl = r.pl;
  return n;
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
  const int s = add_sat(q, d);
  return max(-kPhiQMax, min(kPhiQMax, s));
}

template <bool FIX>
__global__ void __launch_bounds__(32 * kWarps) k_stream_f32(Step2DArgs a) {
  const int lane = threadIdx.x & 31;
  const int strip = blockIdx.x * kWarps + (threadIdx.x >> 5);
  const int x0 = strip * 32;
  if (x0 >= a.Nx) return;  // whole warp leaves together
  const int y0 = blockIdx.y * kRows;
  const int y1 = min(y0 + kRows, a.Ny);
  const int gx = x0 + lane;
  const bool valid = gx < a.Nx;
  const int cx = min(gx, a.Nx - 1);
  // columns outside the strip, handled by lanes 0 (left) and 31 (right)
  const bool edge_lane = lane == 0 || lane == 31;
  const int hx = lane == 0 ? max(x0 - 1, 0) : min(x0 + 32, a.Nx - 1);
  const int P = a.pitch;
  const FastCoef& K = a.k;
  const float idx2 = a.idx2f[0], idy2 = a.idx2f[1];

  auto row_i = [&](int y) { return size_t(min(max(y, 0), a.Ny - 1)) * P; };

  // window: rows y-1 (up), y (c), y+1 (dn)
  Raw<FIX> rc = load_raw<FIX>(a, row_i(y0) + cx);
  Raw<FIX> rdn = load_raw<FIX>(a, row_i(y0 + 1) + cx);
  Nb<FIX> up = solve<FIX>(K, load_raw<FIX>(a, row_i(y0 - 1) + cx));
  Nb<FIX> c = solve<FIX>(K, rc);

  for (int y = y0; y < y1; y++) {
    // prefetch the row after next, and this row's compensation
    const Raw<FIX> rnext = load_raw<FIX>(a, row_i(y + 2) + cx);
    const size_t i = size_t(y) * P + cx;
    const float cin0 = __ldg(a.cin[0] + i), cin1 = __ldg(a.cin[1] + i);
    float cin2 = 0.f, cin3 = 0.f;
    if (!FIX) {
      cin2 = __ldg(a.cin[2] + i);
      cin3 = __ldg(a.cin[3] + i);
    }
    const Nb<FIX> dn = solve<FIX>(K, rdn);
    // the neighbours outside the strip for this row
    Nb<FIX> h{};
    if (edge_lane) h = solve<FIX>(K, load_raw<FIX>(a, size_t(y) * P + hx));

    // horizontal neighbours
    Nb<FIX> w, e;
    w.gcr = __shfl_up_sync(0xffffffffu, c.gcr, 1);
    w.gnb = __shfl_up_sync(0xffffffffu, c.gnb, 1);
    w.pd = __shfl_up_sync(0xffffffffu, c.pd, 1);
    w.pl = __shfl_up_sync(0xffffffffu, c.pl, 1);
    e.gcr = __shfl_down_sync(0xffffffffu, c.gcr, 1);
    e.gnb = __shfl_down_sync(0xffffffffu, c.gnb, 1);
    e.pd = __shfl_down_sync(0xffffffffu, c.pd, 1);
    e.pl = __shfl_down_sync(0xffffffffu, c.pl, 1);
    if (lane == 0) w = h;
    if (lane == 31) e = h;
    // a lane past the domain's right edge holds the edge cell (clamped), so
    // the last valid lane's east neighbour is its mirror already

    // Laplacians: difference form, exact integer differences for FIX phases
    auto lapf = [&](float vw, float ve, float vn, float vs, float vc) {
      const float sx = (vw - vc) + (ve - vc);
      const float sy = (vn - vc) + (vs - vc);
      return fmaf(sx, idx2, sy * idy2);
    };
    const float lapCr = lapf(w.gcr, e.gcr, up.gcr, dn.gcr, c.gcr);
    const float lapNb = lapf(w.gnb, e.gnb, up.gnb, dn.gnb, c.gnb);
    float lapD, lapL;
    if constexpr (FIX) {
      auto lapq = [&](int vw, int ve, int vn, int vs, int vc) {
        const float sx = float(vw - vc) + float(ve - vc);
        const float sy = float(vn - vc) + float(vs - vc);
        return fmaf(sx, idx2, sy * idy2) * kPhiInvScale;
      };
      lapD = lapq(w.pd, e.pd, up.pd, dn.pd, c.pd);
      lapL = lapq(w.pl, e.pl, up.pl, dn.pl, c.pl);
    } else {
      lapD = lapf(w.pd, e.pd, up.pd, dn.pd, c.pd);
      lapL = lapf(w.pl, e.pl, up.pl, dn.pl, c.pl);
    }

    // Cahn-Hilliard with Kahan-compensated accumulation
    const float X = rc.x, Y = rc.y;
    const float incCr = fmaf(a.dtD[0][0], lapCr, a.dtD[0][1] * lapNb);
    const float incNb = fmaf(a.dtD[1][0], lapCr, a.dtD[1][1] * lapNb);
    const float ycr = incCr - cin0, tcr = X + ycr;
    const float ynb = incNb - cin1, tnb = Y + ynb;

    // Allen-Cahn
    const float phd = phf<FIX>(c.pd), phl = phf<FIX>(c.pl);
    const float u1 = c.gcr - K.xe_gam[0], u2 = c.gnb - K.xe_gam[1];
    const float dPd = quad2(K.dP[0], u1, u2), dPl = quad2(K.dP[1], u1, u2);
    const float dFd = -pp32(phd) * dPd + a.om2[0] * phd * (phd - 1.0f) * (2.0f * phd - 1.0f) +
                      a.alpha2 * phd * phl * phl - a.kap[0] * lapD;
    const float dFl = -pp32(phl) * dPl + a.om2[1] * phl * (phl - 1.0f) * (2.0f * phl - 1.0f) +
                      a.alpha2 * phl * phd * phd - a.kap[1] * lapL;

    if (valid) {
      float* const* o = reinterpret_cast<float* const*>(a.out);
      o[0][i] = tcr;
      o[1][i] = tnb;
      a.cout[0][i] = (tcr - X) - ycr;
      a.cout[1][i] = (tnb - Y) - ynb;
      if constexpr (FIX) {
        reinterpret_cast<int*>(o[2])[i] = phi_step(c.pd, -a.dtL[0] * dFd);
        reinterpret_cast<int*>(o[3])[i] = phi_step(c.pl, -a.dtL[1] * dFl);
      } else {
        const float yd = -a.dtL[0] * dFd - cin2, td = phd + yd;
        const float yl = -a.dtL[1] * dFl - cin3, tl = phl + yl;
        o[2][i] = td;
        o[3][i] = tl;
        a.cout[2][i] = (td - phd) - yd;
        a.cout[3][i] = (tl - phl) - yl;
      }
    }
    // slide the window
    up = c;
    c = dn;
    rc = rdn;
    rdn = rnext;
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

}  // namespace

cudaError_t launch_step2d_f32(const Step2DArgs& a, cudaStream_t s) {
  const int strips = (a.Nx + 31) / 32;
  dim3 grid((strips + kWarps - 1) / kWarps, (a.Ny + kRows - 1) / kRows);
  if (a.kahan_phi)
    k_stream_f32<false><<<grid, 32 * kWarps, 0, s>>>(a);
  else
    k_stream_f32<true><<<grid, 32 * kWarps, 0, s>>>(a);
  return cudaGetLastError();
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
