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

// ---- variable-mobility Cahn-Hilliard (FP64) ----
// d2g_<phase>_dx<i><j> as a compile-time constant
template <int PH, int I, int J>
__device__ __forceinline__ constexpr double d2g() {
  return kD2g[PH][I][J];
}

// dg_<phase>_dx<comp>, thermo/parabola625.c:655-706
template <int PH, int C>
__device__ __forceinline__ double dgp64(double X, double Y) {
  constexpr double a = kDgPh[PH][C][0], b = kDgPh[PH][C][1], c = kDgPh[PH][C][2];
  return a * X + b * Y + c;
}

// The composition-dependent diffusivities D_CrCr, D_CrNb, D_NbCr, D_NbNb of
// thermo/parabola625.c:1860-1894, term by term (mobility prefactors times
// the exponentials of the mobility exponents, curvature weights).
__device__ __forceinline__ void dmatrix64(double X, double Y, double D[2][2]) {
  const double xni = -X - Y + 1;
  const double eNb = exp(-34.982563536715503 * Y * xni + 14.437947842988088 * Y);
  const double eCr = exp(-7.1543718172640256 * X * xni + 3.3541967644499233 * X);
  const double eNi = exp(-8.5221193705645018 * X * xni + 4.0036674816806448 * X -
                         442.62877981749585 * Y * xni - 0.82164267100913768 * Y);
  const double s0 = -kHCrCr * X - kHCrNb * Y;  // curvature row of the Cr column
  const double s1 = -kHCrNb * X - kHNbNb * Y;  // of the Nb column
  D[0][0] = -kMobPreNb * X * Y * (s0 + kHCrNbAddA) * eNb + kMobPreCr * X * (1 - X) * (s0 + kHCrCrAdd) * eCr -
            kMobPreNi * X * s0 * xni * eNi;
  D[0][1] = -kMobPreNb * X * Y * (s1 + kHNbNbAdd) * eNb + kMobPreCr * X * (1 - X) * (s1 + kHCrNbAddB) * eCr -
            kMobPreNi * X * s1 * xni * eNi;
  D[1][0] = -kMobPreCr * X * Y * (s0 + kHCrCrAdd) * eCr + kMobPreNb * Y * (1 - Y) * (s0 + kHCrNbAddA) * eNb -
            kMobPreNi * Y * s0 * xni * eNi;
  D[1][1] = -kMobPreCr * X * Y * (s1 + kHCrNbAddB) * eCr + kMobPreNb * Y * (1 - Y) * (s1 + kHNbNbAdd) * eNb -
            kMobPreNi * Y * s1 * xni * eNi;
}

// The 16 coefficients of the variable-mobility flux at one cell (the
// reference's disabled mobility_Cr_kernel / mobility_Nb_kernel,
// src/discretization.cu:175-296).  The reference never defines the mobility
// matrix those kernels call; here M = D(x) H_gam^-1 (H_gam the gamma
// curvatures), so that in pure gamma the flux is D(x) grad x^gamma.
// o[0..7]: Cr row gam_CrCr gam_CrNb del_CrCr del_CrNb lav_CrCr lav_CrNb
// phi_del_Cr phi_lav_Cr; o[8..15] the Nb row likewise.  xg, xd, xl: the
// cell's fictitious compositions (Cr, Nb).
__device__ __forceinline__ void mobility64(double X, double Y, double phd, double phl, double pD,
                                           double pG, double pL, const double xg[2],
                                           const double xd[2], const double xl[2], double o[16]) {
  constexpr double hg00 = d2g<0, 0, 0>(), hg01 = d2g<0, 0, 1>(), hg10 = d2g<0, 1, 0>(),
                   hg11 = d2g<0, 1, 1>();
  constexpr double det = hg00 * hg11 - hg01 * hg10;
  double D[2][2];
  dmatrix64(X, Y, D);
  double M[2][2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    M[k][0] = (D[k][0] * hg11 - D[k][1] * hg10) / det;
    M[k][1] = (D[k][1] * hg00 - D[k][0] * hg01) / det;
  }
  const double dgg0 = dgp64<0, 0>(xg[0], xg[1]), dgg1 = dgp64<0, 1>(xg[0], xg[1]);
  const double dgd0 = dgp64<1, 0>(xd[0], xd[1]) - dgg0, dgd1 = dgp64<1, 1>(xd[0], xd[1]) - dgg1;
  const double dgl0 = dgp64<2, 0>(xl[0], xl[1]) - dgg0, dgl1 = dgp64<2, 1>(xl[0], xl[1]) - dgg1;
  const double ppd = pp64(phd), ppl = pp64(phl);
  // Cr row (mobility_Cr_kernel, terms 1-8)
  o[0] = pG * (M[0][0] * d2g<0, 0, 0>() + M[0][1] * d2g<0, 0, 1>());
  o[1] = pG * (M[0][0] * d2g<0, 1, 0>() + M[0][1] * d2g<0, 1, 1>());
  o[2] = pD * (M[0][0] * d2g<1, 0, 0>() + M[0][1] * d2g<1, 0, 1>());
  o[3] = pD * (M[0][0] * d2g<1, 1, 0>() + M[0][1] * d2g<1, 1, 1>());
  o[4] = pL * (M[0][0] * d2g<2, 0, 0>() + M[0][1] * d2g<2, 0, 1>());
  o[5] = pL * (M[0][0] * d2g<2, 1, 0>() + M[0][1] * d2g<2, 1, 1>());
  o[6] = ppd * (M[0][0] * dgd0 + M[0][1] * dgd1);
  o[7] = ppl * (M[0][0] * dgl0 + M[0][1] * dgl1);
  // Nb row (mobility_Nb_kernel: its terms 1-6 read d2g_..._dxNbCr where the
  // Cr kernel reads ..._dxCrNb -- equal, the curvature matrices are symmetric)
  o[8] = pG * (M[1][0] * d2g<0, 0, 0>() + M[1][1] * d2g<0, 1, 0>());
  o[9] = pG * (M[1][0] * d2g<0, 1, 0>() + M[1][1] * d2g<0, 1, 1>());
  o[10] = pD * (M[1][0] * d2g<1, 0, 0>() + M[1][1] * d2g<1, 1, 0>());
  o[11] = pD * (M[1][0] * d2g<1, 1, 0>() + M[1][1] * d2g<1, 1, 1>());
  o[12] = pL * (M[1][0] * d2g<2, 0, 0>() + M[1][1] * d2g<2, 1, 0>());
  o[13] = pL * (M[1][0] * d2g<2, 1, 0>() + M[1][1] * d2g<2, 1, 1>());
  o[14] = ppd * (M[1][0] * dgd0 + M[1][1] * dgd1);
  o[15] = ppl * (M[1][0] * dgl0 + M[1][1] * dgl1);
}

// discrete_laplacian, src/discretization.cu:605-616: the 1D difference of a
// variable coefficient D times the gradient of c; r2 = 1 / (2 d^2)
__device__ __forceinline__ double dlap64(double Dl, double Dm, double Dh, double cl, double cm,
                                         double ch, double r2) {
  return ((Dh + Dm) * (ch - cm) - (Dm + Dl) * (cm - cl)) * r2;
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

// The diffusivity matrix D(X, Y) of dmatrix64 (thermo/parabola625.c:1860-1894)
// in FP32, with the mobility prefactors (Nb, Cr, Ni) passed in `pre` already
// multiplied by a scale the caller chooses (dt / (2 dx^2) in the FP32
// variable-mobility step, which keeps the entries near 1e-4 .. 1e-1).  The
// mobility exponents are at most 14.5 on the composition simplex, so no
// exponential overflows; a term whose exponential underflows is negligible.
// __expf is within 2 + 1.17 |x| ulp: 2e-6 relative for the exponents of the
// terms that matter (|x| < 15), against the 1e-5 the FP32 step is held to.
__device__ __forceinline__ void dmat32(const float pre[3], float X, float Y, float& d00,
                                       float& d01, float& d10, float& d11) {
  const float xni = 1.0f - X - Y;
  const float eNb = pre[0] * __expf(fmaf(-34.982563536715503f * Y, xni, 14.437947842988088f * Y));
  const float eCr = pre[1] * __expf(fmaf(-7.1543718172640256f * X, xni, 3.3541967644499233f * X));
  const float eNi = pre[2] * __expf(fmaf(-8.5221193705645018f * X, xni, 4.0036674816806448f * X) -
                                  fmaf(442.62877981749585f * Y, xni, 0.82164267100913768f * Y));
  const float s0 = -float(kHCrCr) * X - float(kHCrNb) * Y;  // curvature row of the Cr column
  const float s1 = -float(kHCrNb) * X - float(kHNbNb) * Y;  // of the Nb column
  const float xy = X * Y, xx = X * (1.0f - X), yy = Y * (1.0f - Y);
  const float niX = eNi * X * xni, niY = eNi * Y * xni;
  d00 = -eNb * xy * (s0 + float(kHCrNbAddA)) + eCr * xx * (s0 + float(kHCrCrAdd)) - niX * s0;
  d01 = -eNb * xy * (s1 + float(kHNbNbAdd)) + eCr * xx * (s1 + float(kHCrNbAddB)) - niX * s1;
  d10 = -eCr * xy * (s0 + float(kHCrCrAdd)) + eNb * yy * (s0 + float(kHCrNbAddA)) - niY * s0;
  d11 = -eCr * xy * (s1 + float(kHCrNbAddB)) + eNb * yy * (s1 + float(kHNbNbAdd)) - niY * s1;
}

// c0 + a (c1 + c11 a + c12 b) + b (c2 + c22 b), coefficients in the order
// c0 c1 c2 c11 c12 c22
__device__ __forceinline__ float quad2(const float* c, float a, float b) {
  return fmaf(a, fmaf(c[3], a, fmaf(c[4], b, c[1])), fmaf(b, fmaf(c[5], b, c[2]), c[0]));
}

// ---- FP32 form: values in FP32, Kahan compensations c (value = hi - c) ----
// Packed compensation record: four 16-bit counts, c = count 2^-40 for the
// compositions and count 2^-39 for the phases.  A compensation is at most
// half an ulp of its value -- below 2^-25 for |x| < 1 and 2^-24 for
// |phi| < 2 -- so the counts keep 2^-40 (2^-39) of resolution, and a field
// loses at most half of that per step where the full FP32 compensation
// would keep it.
constexpr float kCqX = 1099511627776.0f;  // 2^40
constexpr float kCqP = 549755813888.0f;   // 2^39
constexpr float kCqXi = 1.0f / 1099511627776.0f;
constexpr float kCqPi = 1.0f / 549755813888.0f;

// Two counts (values already scaled) as the 16-bit halves of one word: cvt's
// float-to-integer conversion rounds to nearest even and saturates to
// [-32768, 32767] in one instruction per half.
__device__ __forceinline__ unsigned cq_pair(float lo, float hi) {
  unsigned r;
  asm("{\n\t.reg .s16 l, h;\n\tcvt.rni.s16.f32 l, %1;\n\tcvt.rni.s16.f32 h, %2;\n\t"
      "mov.b32 %0, {l, h};\n\t}"
      : "=r"(r)
      : "f"(lo), "f"(hi));
  return r;
}

// the two signed 16-bit halves of a word as FP32 (exact)
__device__ __forceinline__ float2 cq_halves(unsigned w) {
  float2 f;
  asm("{\n\t.reg .s16 l, h;\n\tmov.b32 {l, h}, %2;\n\tcvt.rn.f32.s16 %0, l;\n\t"
      "cvt.rn.f32.s16 %1, h;\n\t}"
      : "=f"(f.x), "=f"(f.y)
      : "r"(w));
  return f;
}

__device__ __forceinline__ float4 cq_unpack(uint2 w) {
  const float2 a = cq_halves(w.x), b = cq_halves(w.y);
  return make_float4(a.x * kCqXi, a.y * kCqXi, b.x * kCqPi, b.y * kCqPi);
}

// one compensation as its 16-bit count (the halves cq_pair writes)
__device__ __forceinline__ unsigned cq_count(float c, float scale) {
  return cq_pair(c * scale, 0.0f) & 0xffffu;
}

__device__ __forceinline__ uint2 cq_pack(float cx, float cy, float cd, float cl) {
  return make_uint2(cq_pair(cx * kCqX, cy * kCqX), cq_pair(cd * kCqP, cl * kCqP));
}

// 1 - p(x) = p(1 - x): the gamma fraction without cancellation near a pure
// precipitate (1 - phi is exact in FP32 for phi >= 1/2).
__device__ __forceinline__ float p_gamma32(float phd, float phl, float pD, float pL) {
  return pD >= pL ? p32(1.0f - phd) - pL : p32(1.0f - phl) - pD;
}

// Phases below this (both fields) leave p(phi) < 1e-14: x^gamma = X to FP64
// precision.
constexpr float kBulkPhi = 1e-5f;

// u = x^gamma - xe_gamma in pure gamma: X - xe_gamma, X = hi - c.
__device__ __forceinline__ void gamma_bulk32(const FastCoef& K, float X, float Y, float cx,
                                             float cy, float& u1, float& u2) {
  u1 = (X - K.xe_hi[0][0]) - (cx + K.xe_lo[0][0]);
  u2 = (Y - K.xe_hi[0][1]) - (cy + K.xe_lo[0][1]);
}

// u = x^gamma - xe_gamma of one cell in the equilibrium-referenced form
// (FastCoef): u = d + (A d_Cr + B d_Nb) / den, d = X - X*(p).  X* is
// expanded about the phase with the largest p (the pivot m):
//   X* = xe_m + sum_{i != m} p_i xe_i - (sum_{i != m} p_i) xe_m,
// and d = (hi - xe_m,hi) - (c + xe_m,lo + that sum), so the leading
// difference is exact where X is near the pivot's composition and every
// other term is small there (approximate reciprocal: 2 ulp).
__device__ __forceinline__ void gamma_u32(const FastCoef& K, float X, float Y, float cx, float cy,
                                          float phd, float phl, float& u1, float& u2) {
  const float pD = p32(phd), pL = p32(phl);
  const float pG = p_gamma32(phd, phl, pD, pL);
  const int piv = (pG >= pD && pG >= pL) ? 0 : (pD >= pL ? 1 : 2);
  const float t0 = piv == 0 ? 0.0f : pG, t1 = piv == 1 ? 0.0f : pD, t2 = piv == 2 ? 0.0f : pL;
  const float s = t0 + t1 + t2;
  const float xv[2] = {X, Y}, cv[2] = {cx, cy};
  float dv[2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const float xh = piv == 0 ? K.xe_hi[0][k] : (piv == 1 ? K.xe_hi[1][k] : K.xe_hi[2][k]);
    const float xl = piv == 0 ? K.xe_lo[0][k] : (piv == 1 ? K.xe_lo[1][k] : K.xe_lo[2][k]);
    const float mix =
        fmaf(t0, K.xe_hi[0][k], fmaf(t1, K.xe_hi[1][k], fmaf(t2, K.xe_hi[2][k], -s * xh)));
    dv[k] = (xv[k] - xh) - (cv[k] + xl + mix);
  }
  const float m[5] = {pD * pD, pD * pG, pD * pL, pG * pL, pL * pL};
  const float* d = K.den;
  const float den = fmaf(d[0], m[0], fmaf(d[1], m[1], fmaf(d[2], m[2], fmaf(d[3], pG * pG, fmaf(d[4], m[3], d[5] * m[4])))));
  const float r = __fdividef(1.0f, den);
  float u[2];
#pragma unroll
  for (int c = 0; c < 2; c++) {
    float a = 0.0f, b = 0.0f;
#pragma unroll
    for (int j = 0; j < 5; j++) {
      a = fmaf(K.dev[c][j][0], m[j], a);
      b = fmaf(K.dev[c][j][1], m[j], b);
    }
    u[c] = fmaf(fmaf(a, dv[0], b * dv[1]), r, dv[c]);
  }
  u1 = u[0];
  u2 = u[1];
}

// dF/dphi_i without the Laplacian term: -p'(phi) dP + 2 omega phi (phi-1)(2 phi-1)
// + 2 alpha phi phi_j^2, Horner forms
__device__ __forceinline__ float dF_local32(float ph, float pj, float dP, float om2,
                                            float alpha2) {
  const float t = fmaf(-ph, ph, ph);  // phi (1 - phi)
  const float pp = 30.0f * t * t;     // p'(phi)
  const float well = ph * fmaf(ph, fmaf(2.0f * om2, ph, -3.0f * om2), om2);
  return fmaf(-pp, dP, fmaf(alpha2 * ph, pj * pj, well));
}

// hi = the FP32 value nearest v and c = float(double(hi) - v): the split of
// the FP32 form (value = hi - c), computed from the bits of v without FP64
// arithmetic (this part issues FP64 at ~1/64 of the FP32 rate, and the
// conversions would bound the layout conversion kernels).  For 950 <= E <=
// 1149 (E: v's biased exponent) hi and c are FP32-normal and double(hi) - v
// = -rem 2^(E-1075) is exact with |rem| <= 2^28, so rounding -rem to FP32
// and scaling by the power of two gives the FP64 expression's result
// bit-for-bit; zeros take hi = v, c = +0; every other double takes the FP64
// expression itself.
__device__ __forceinline__ void split_f64(double v, float& hi, float& c) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
  const int E = int((b >> 52) & 0x7ff);
  const unsigned sign = unsigned(b >> 32) & 0x80000000u;
  if ((b << 1) == 0ull) {
    hi = __int_as_float(int(sign));
    c = 0.0f;
    return;
  }
  if (E < 950 || E > 1149) {
    hi = float(v);
    c = float(double(hi) - v);
    return;
  }
  const unsigned long long M = (b & 0xfffffffffffffull) | (1ull << 52);
  unsigned q = unsigned(M >> 29);  // the 24 leading bits
  int rem = int(M & 0x1fffffffull);  // the 29 dropped bits
  if (rem > (1 << 28) || (rem == (1 << 28) && (q & 1u))) {  // round to nearest even
    q += 1u;
    rem -= 1 << 29;
  }
  // q = 2^24 carries into the exponent field
  hi = __int_as_float(int(sign | ((unsigned(E - 896) << 23) + (q - (1u << 23)))));
  const float scale = __int_as_float((E - 1075 + 127) << 23);
  // c = hi - v = -rem 2^(E-1075) for v > 0, +rem 2^(E-1075) for v < 0
  // (rem = 0 gives +0, as the FP64 subtraction does)
  c = __int2float_rn(sign ? rem : -rem) * scale;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with
// Weyl-sequence key bumps (nucleation draws, initial-condition noise).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
  constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    if (r > 0) {
      k.x += W0;
      k.y += W1;
    }
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
  }
  return c;
}

// 53 random bits -> uniform double in (0, 1]
__device__ __forceinline__ double u53(uint32_t hi, uint32_t lo) {
  const unsigned long long k = ((((unsigned long long)hi) << 32) | lo) >> 11;
  return double(k + 1ull) * (1.0 / 9007199254740992.0);
}

}  // namespace dev
}  // namespace pfa
