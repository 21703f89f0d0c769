// pfa_device.cuh -- device-side model functions of libpfa_gb300.
//
// FP64 functions follow the reference's generated formulas term by term
// (thermo/parabola625.c; device copies src/parabola625.cu) so that the plain
// FP64 step stays within 1e-12 of the reference.  FP32 helpers evaluate the
// reduced forms whose coefficients pfa_model.cpp derives (pfa::FastCoef).
#pragma once

#include <cuda_runtime.h>

#include "pfa_internal.h"
#include "pfa_model.h"

namespace pfa {
namespace dev {

// p(x) = x^3 (6x^2 - 15x + 10), thermo/parabola625.c:11-18
__device__ __forceinline__ double p64(double x) {
  const double x2 = x * x;
  return x2 * x * (6.0 * x2 - 15.0 * x + 10.0);
}

// p'(x) = 30 x^2 (1 - x)^2, thermo/parabola625.c:20-27
__device__ __forceinline__ double pp64(double x) {
  const double y = 1.0 - x;
  return 30.0 * (x * x) * (y * y);
}

// Shared pieces of the six fictitious compositions at one cell.
struct Poly64 {
  double lin[3];   // pDel, pGam, pLav
  double mono[6];  // pD^2, pD pG, pD pL, pG^2, pG pL, pL^2
  double rden;     // 1 / shared denominator
};

__device__ __forceinline__ void poly64(double pD, double pG, double pL, Poly64& m) {
  m.lin[0] = pD;
  m.lin[1] = pG;
  m.lin[2] = pL;
  m.mono[0] = pD * pD;
  m.mono[1] = pD * pG;
  m.mono[2] = pD * pL;
  m.mono[3] = pG * pG;
  m.mono[4] = pG * pL;
  m.mono[5] = pL * pL;
  constexpr double d0 = kDen[0], d1 = kDen[1], d2 = kDen[2], d3 = kDen[3], d4 = kDen[4],
                   d5 = kDen[5];
  const double den = d0 * m.mono[0] + d1 * m.mono[1] + d2 * m.mono[2] + d3 * m.mono[3] +
                     d4 * m.mono[4] + d5 * m.mono[5];
  m.rden = 1.0 / den;
}

// fict_<phase>_<comp>, thermo/parabola625.c:245-297
template <int PH, int C>
__device__ __forceinline__ double fict64(double X, double Y, const Poly64& m) {
  constexpr FictRow r = kFict[PH][C];
  const double lx = r.l[0] * m.lin[0] + r.l[1] * m.lin[1] + r.l[2] * m.lin[2];
  const double ly = r.m[0] * m.lin[0] + r.m[1] * m.lin[1] + r.m[2] * m.lin[2];
  const double q = r.q[0] * m.mono[0] + r.q[1] * m.mono[1] + r.q[2] * m.mono[2] +
                   r.q[3] * m.mono[3] + r.q[4] * m.mono[4] + r.q[5] * m.mono[5];
  return (r.scale * (X * lx + Y * ly + q)) * m.rden;
}

// g_<phase>, thermo/parabola625.c:418-443
template <int PH>
__device__ __forceinline__ double g64(double X, double Y) {
  constexpr double A = kG[PH][0], B = kG[PH][1], Cc = kG[PH][2], E = kG[PH][3];
  constexpr double x0 = kXe[PH][0], y0 = kXe[PH][1];
  const double u = X - x0, v = Y - y0;
  return A * (u * u) + (B * X - Cc) * v + E * (v * v);
}

// dg_gam_dx<comp>, thermo/parabola625.c:655-671
template <int C>
__device__ __forceinline__ double dg64(double X, double Y) {
  constexpr double a = kDg[C][0], b = kDg[C][1], c = kDg[C][2];
  return a * X + b * Y + c;
}

// ---- FP32 fast forms ----
__device__ __forceinline__ float p32(float x) {
  const float x2 = x * x;
  return x2 * x * fmaf(fmaf(6.0f, x, -15.0f), x, 10.0f);
}

__device__ __forceinline__ float pp32(float x) {
  const float y = 1.0f - x;
  return 30.0f * (x * x) * (y * y);
}

// c0 + a (c1 + c11 a + c12 b) + b (c2 + c22 b), coefficients in the order
// c0 c1 c2 c11 c12 c22
__device__ __forceinline__ float quad2(const float* c, float a, float b) {
  return fmaf(a, fmaf(c[3], a, fmaf(c[4], b, c[1])), fmaf(b, fmaf(c[5], b, c[2]), c[0]));
}

// ---- fixed-point phase fields of the FP32 form: phi = q 2^-29 ----
// Resolution 1.9e-9 everywhere on [-1.99, 1.99] (FP32 has 6e-8 near
// phi = 1), so Allen-Cahn increments far below FP32's half-ulp still move
// the field; q is saturated so that the difference of two values fits int32.
constexpr float kPhiScale = 536870912.0f;  // 2^29
constexpr float kPhiInvScale = 1.0f / 536870912.0f;
constexpr double kPhiInvScaleD = 1.0 / 536870912.0;
constexpr int kPhiQMax = 1068373114;  // floor(1.99 * 2^29)

__device__ __forceinline__ float phi_of(int q) { return float(q) * kPhiInvScale; }

__device__ __forceinline__ int phi_sat(long long q) {
  return int(q > kPhiQMax ? kPhiQMax : (q < -kPhiQMax ? -kPhiQMax : q));
}

// q + round(inc 2^29), saturated (the increment is clamped first so its
// integer form cannot overflow)
__device__ __forceinline__ int phi_add(int q, float inc) {
  const float c = fminf(fmaxf(inc, -3.9f), 3.9f);
  return phi_sat((long long)q + __float2int_rn(c * kPhiScale));
}

__device__ __forceinline__ int phi_quantize(double v) {
  const double c = fmin(fmax(v, -1.99), 1.99);
  return phi_sat(__double2ll_rn(c * 536870912.0));
}

// 1 - p(x) = p(1 - x): the gamma fraction without cancellation near a pure
// precipitate (1 - phi is exact in FP32 for phi >= 1/2).
__device__ __forceinline__ float p_gamma32(float phd, float phl, float pD, float pL) {
  return pD >= pL ? p32(1.0f - phd) - pL : p32(1.0f - phl) - pD;
}

// x^gamma (Cr, Nb) from (X, Y, pD, pG, pL), three-variable form.
__device__ __forceinline__ void fict_gam32(const FastCoef& k, float X, float Y, float pD, float pG,
                                           float pL, float& gcr, float& gnb) {
  const float m0 = pD * pD, m1 = pD * pG, m2 = pD * pL, m3 = pG * pG, m4 = pG * pL, m5 = pL * pL;
  const float* d = k.den;
  const float den = fmaf(d[0], m0, fmaf(d[1], m1, fmaf(d[2], m2, fmaf(d[3], m3, fmaf(d[4], m4, d[5] * m5)))));
  const float r = __frcp_rn(den);
  float n[2];
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const float* a = k.num[c];
    const float lx = fmaf(a[0], pD, fmaf(a[1], pG, a[2] * pL));
    const float ly = fmaf(a[3], pD, fmaf(a[4], pG, a[5] * pL));
    const float q = fmaf(a[6], m0, fmaf(a[7], m1, fmaf(a[8], m2, fmaf(a[9], m3, fmaf(a[10], m4, a[11] * m5)))));
    n[c] = fmaf(X, lx, fmaf(Y, ly, q));
  }
  gcr = n[0] * r;
  gnb = n[1] * r;
}

}  // namespace dev
}  // namespace pfa
