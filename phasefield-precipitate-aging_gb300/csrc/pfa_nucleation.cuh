// pfa_nucleation.cuh -- device helpers of the nucleation kernels (sm_103a):
// value access, the reference's probability, the FP32 screen, the FP64
// decision and the event lists.  Included by .cu files only.
#pragma once

#include <cmath>
#include <cstdint>

#include "pfa_device.cuh"
#include "pfa_nucleation.h"

namespace pfa {
namespace {

using namespace dev;

// the screen's margin (nats) over its FP32 evaluation error, and the bound
// on ln z below which no draw is needed (ln 2^-56)
constexpr float kNucMargin = 2.0f;
constexpr float kNucNoDraw = -38.8f;

template <class T>
__device__ __forceinline__ double ld(const void* p, size_t i) {
  return double(static_cast<const T*>(p)[i]);
}

// Storage index of reference cell (xx, yy, zz) (ghost-ring coordinates; zz
// = 0 in 2D).  The FP32 form stores the interior only: a ghost cell reads its
// mirror.
__device__ __forceinline__ size_t stor(const NucArgs& a, int xx, int yy, int zz = 0) {
  if (a.compact) {
    const int cx = min(max(xx - 1, 0), a.Nx - 1), cy = min(max(yy - 1, 0), a.Ny - 1);
    const int cz = a.is3d ? min(max(zz - 1, 0), a.Nz - 1) : 0;
    return (size_t(cz) * a.Ny + cy) * a.pitch + cx;
  }
  return (size_t(zz) * (a.Ny + 2) + yy) * a.pitch + xx;
}

// Kahan compensation of field k at a cell of the FP32 form (value = f - c)
__device__ __forceinline__ float comp_get(const NucArgs& a, size_t cell, int k) {
  if (!a.comp) return 0.0f;
  float4 c;
  if (a.pack)
    c = cq_unpack(static_cast<const uint2*>(a.comp)[cell]);
  else
    c = static_cast<const float4*>(a.comp)[cell];
  return k == 0 ? c.x : (k == 1 ? c.y : (k == 2 ? c.z : c.w));
}

__device__ __forceinline__ void comp_set(const NucArgs& a, size_t cell, int k, float c) {
  if (!a.comp) return;
  if (a.pack)
    static_cast<short*>(a.comp)[4 * cell + k] = short(cq_count(c, k < 2 ? kCqX : kCqP));
  else
    static_cast<float*>(a.comp)[4 * cell + k] = c;
}

// a field's value as stored (FP64, or the FP32 form's hi - c), exact
template <class T>
__device__ __forceinline__ double ldval(const NucArgs& a, int k, size_t cell) {
  return ld<T>(a.f[k], cell * a.stride) - double(comp_get(a, cell, k));
}

// a phase field rounded to FP32 without touching the FP64 pipe in the FP32 form
template <class T>
__device__ __forceinline__ float ldphi_f(const NucArgs& a, int k, size_t cell) {
  return float(static_cast<const T*>(a.f[k])[cell * a.stride]);
}

// the four fields of one cell as stored, rounded to FP32 (x_Cr, x_Nb,
// phi_del, phi_lav): one 16-byte record in the FP32 form, four loads from
// the four FP64 arrays otherwise
template <class T>
__device__ __forceinline__ void own_values(const NucArgs& a, size_t s, float v[4]) {
  if constexpr (sizeof(T) == 4) {
    if (a.stride == 4) {
      const float4 r = static_cast<const float4*>(a.f[0])[s];
      v[0] = r.x;
      v[1] = r.y;
      v[2] = r.z;
      v[3] = r.w;
      return;
    }
  }
#pragma unroll
  for (int k = 0; k < 4; k++) v[k] = float(static_cast<const T*>(a.f[k])[s * a.stride]);
}

// composition-dependent diffusivities D_CrCr, D_NbNb (thermo/parabola625.c:1860-1894)
__device__ void diffusivities(double X, double Y, double& dcc, double& dnn) {
  const double xni = -X - Y + 1;
  const double mNb = kMobPreNb * exp(-34.982563536715503 * Y * xni + 14.437947842988088 * Y);
  const double mCr = kMobPreCr * exp(-7.1543718172640256 * X * xni + 3.3541967644499233 * X);
  const double mNi = kMobPreNi * exp(-8.5221193705645018 * X * xni + 4.0036674816806448 * X -
                                     442.62877981749585 * Y * xni - 0.82164267100913768 * Y);
  const double s0 = -kHCrCr * X - kHCrNb * Y;  // column Cr
  const double s1 = -kHCrNb * X - kHNbNb * Y;  // column Nb
  dcc = -mNb * X * Y * (s0 + kHCrNbAddA) + mCr * X * (1 - X) * (s0 + kHCrCrAdd) - mNi * X * s0 * xni;
  dnn = -mCr * X * Y * (s1 + kHCrNbAddB) + mNb * Y * (1 - Y) * (s1 + kHNbNbAdd) - mNi * Y * s1 * xni;
}

// nucleation_probability_sphere, thermo/nucleation.c:30-69 (src/nucleation.cu:30-70)
__device__ void probability_sphere(double xCr, double xNb, double dG, double dcc, double dnn,
                                   double sigma, double Vatom, double n_gam, double dV, double dt,
                                   double& Rstar, double& P) {
  const double sigma_cubed = sigma * sigma * sigma;
  const double Zeldov = (Vatom * dG * dG) / (8. * kPi * sqrt(kKT * sigma_cubed));
  const double Gstar = (16. * kPi * sigma_cubed) / (3. * dG * dG);
  constexpr double a2 = kLatticeConst * kLatticeConst;
  const double a4 = a2 * a2;
  const double BstarCr = (3. * Gstar * dcc * xCr) / (sigma * a4);
  const double BstarNb = (3. * Gstar * dnn * xNb) / (sigma * a4);
  const double k1Cr = BstarCr * Zeldov * n_gam;
  const double k1Nb = BstarNb * Zeldov * n_gam;
  const double k2 = Gstar / kKT;
  const double dc_Cr = -xCr + kXe[0][0];
  const double dc_Nb = xNb - kXe[0][1];
  const double JCr = k1Cr * exp(-k2 / dc_Cr);
  const double JNb = k1Nb * exp(-k2 / dc_Nb);
  const double P0 = exp(-dt * dV * (JCr + JNb));
  P = 1. - P0;
  Rstar = (2. * sigma) / dG;
}

// Upper bound, in FP32, of ln z with z = dt dV (J_Cr + J_Nb) for each phase
// (thermo/nucleation.c:30-69): J_k = k1_k exp(-k2 / dc_k) with
//   k1_k = 3 G* D_kk x_k Zeldovich n_gam / (sigma a^4),  k2 = G* / kT,
// G* = 16 pi sigma^3 / (3 dG^2) and Zeldovich ~ dG^2, so the dG factors of
// k1 cancel: ln k1_k = lnK + ln(D_kk x_k) with the per-phase constant lnK
// of the host (NucArgs, ln(dt dV) included) and k2 = C2 / dG^2.  Two tiers:
//  1. (ln_z_tier1) without transcendentals: |D_kk| <= 3 x 1.5e-20 exp(max e)
//     x 2.5e6 (prefactors, |s| + add; e the mobility exponents) and x <= 1,
//       ln z <= lnC1 + max e - k2 / max_k dc_k     (lnC1 = lnK + ln 2 + that bound);
//     this settles most of the matrix;
//  2. (ln_z_tier2) D_kk evaluated in FP32 with a bound on its error (every
//     term to 1e-3 of its magnitude, plus 1e-30 for terms that underflow):
//     a term whose D_kk is certainly <= 0 has J_k <= 0 and adds nothing;
//     where both are, or where a certainly negative term outweighs the other
//     term's upper bound by 0.25 nats, z <= 0 and no draw can make an event
//     (-inf); otherwise z <= 2 dt dV max_k k1_k+ exp(-k2 / dc_k).
// Each tier is an upper bound.  +inf where no bound is attempted
// (compositions outside the simplex, or at or above the gamma equilibrium
// composition, where the exponents change sign, or dG <= 1).
struct ZPre {
  float dcCr, dcNb, inv2, eNb, eCr, eNi;
  bool ok;
};

__device__ __forceinline__ ZPre z_pre(float X, float Y) {
  constexpr float xgCr = float(kXe[0][0]), xgNb = float(kXe[0][1]);
  ZPre p;
  p.dcCr = xgCr - X;
  p.dcNb = Y - xgNb;
  p.ok = p.dcCr > 0.0f && p.dcNb > 0.0f && X > 0.0f && Y > 0.0f && X + Y < 1.0f;
  const float u = X - xgCr, v = Y - xgNb;
  const float dG = float(kG[0][0]) * u * u + (float(kG[0][1]) * X - float(kG[0][2])) * v +
                   float(kG[0][3]) * v * v;
  p.ok = p.ok && dG > 1.0f;
  p.inv2 = __fdividef(1.0f, dG * dG);
  const float xni = 1.0f - X - Y;
  p.eNb = -34.982563536715503f * Y * xni + 14.437947842988088f * Y;
  p.eCr = -7.1543718172640256f * X * xni + 3.3541967644499233f * X;
  p.eNi = -8.5221193705645018f * X * xni + 4.0036674816806448f * X -
          442.62877981749585f * Y * xni - 0.82164267100913768f * Y;
  return p;
}

__device__ __forceinline__ void ln_z_tier1(const ZPre& p, const NucArgs& a, float lnz[2]) {
  lnz[0] = lnz[1] = INFINITY;
  if (!p.ok) return;
  const float emax = fmaxf(p.eNb, fmaxf(p.eCr, p.eNi));
  const float inv = __fdividef(p.inv2, fmaxf(p.dcCr, p.dcNb));
#pragma unroll
  for (int ph = 0; ph < 2; ph++) {
    const float l = a.lnC1[ph] + emax - a.C2[ph] * inv;
    if (l == l) lnz[ph] = l;  // NaN stays +inf
  }
}

// tier 2 (p.ok): lnz[] holds tier 1's bounds on entry; the smaller is kept
__device__ __forceinline__ void ln_z_tier2(float X, float Y, const ZPre& p, const NucArgs& a,
                                           float lnz[2]) {
  // the diffusivities of thermo/parabola625.c:1860-1894 in FP32.  The fast
  // exponential and logarithm suffice: __expf is within 2 + 1.17 |x| ulp
  // (6e-6 relative at |x| = 44), far inside the 1e-3 relative slack added to
  // each sum below, and __logf within 2^-21 absolute, far inside the 0.25 and
  // kNucMargin nats the bounds carry; exponents below -87 flush to 0 where
  // expf would give a subnormal, which the 1e-30 floor of each sum covers.
  const float xni = 1.0f - X - Y;
  const float mNb = float(kMobPreNb) * __expf(p.eNb);
  const float mCr = float(kMobPreCr) * __expf(p.eCr);
  const float mNi = float(kMobPreNi) * __expf(p.eNi);
  const float s0 = -float(kHCrCr) * X - float(kHCrNb) * Y;
  const float s1 = -float(kHCrNb) * X - float(kHNbNb) * Y;
  const float t0 = -mNb * X * Y * (s0 + float(kHCrNbAddA));
  const float t1 = mCr * X * (1.0f - X) * (s0 + float(kHCrCrAdd));
  const float t2 = -mNi * X * s0 * xni;
  const float q0 = -mCr * X * Y * (s1 + float(kHCrNbAddB));
  const float q1 = mNb * Y * (1.0f - Y) * (s1 + float(kHNbNbAdd));
  const float q2 = -mNi * Y * s1 * xni;
  const float dcc_up = (t0 + t1 + t2) + 1e-3f * (fabsf(t0) + fabsf(t1) + fabsf(t2)) + 1e-30f;
  const float dnn_up = (q0 + q1 + q2) + 1e-3f * (fabsf(q0) + fabsf(q1) + fabsf(q2)) + 1e-30f;
  if (!(dcc_up > 0.0f) && !(dnn_up > 0.0f)) {
    if (dcc_up == dcc_up && dnn_up == dnn_up) lnz[0] = lnz[1] = -INFINITY;
    return;
  }
  // ln of |D_kk| x_k: the positive part's upper bound, or the magnitude's
  // lower bound where the upper bound is negative
  const float lDX = __logf(fabsf(dcc_up) * X), lDY = __logf(fabsf(dnn_up) * Y);
  const float rCr = __fdividef(1.0f, p.dcCr), rNb = __fdividef(1.0f, p.dcNb);
#pragma unroll
  for (int ph = 0; ph < 2; ph++) {
    const float k2 = a.C2[ph] * p.inv2;
    const float lCr = lDX - k2 * rCr, lNb = lDY - k2 * rNb;
    const float upCr = dcc_up > 0.0f ? lCr : -INFINITY;
    const float upNb = dnn_up > 0.0f ? lNb : -INFINITY;
    if ((dcc_up < 0.0f && lCr > upNb + 0.25f) || (dnn_up < 0.0f && lNb > upCr + 0.25f)) {
      lnz[ph] = -INFINITY;
      continue;
    }
    // the sum of two terms is at most twice the larger
    const float l = fmaxf(upCr, upNb) + a.lnK[ph] + 0.69314718f;
    if (l == l) lnz[ph] = fminf(lnz[ph], l);
  }
}

// p(phi_del) + p(phi_lav) < 1e-10 as the reference's FP64 test decides it:
// in FP32 when the FP32 sum is farther from the threshold than its error
// bound (1e-6 of |p_del| + |p_lav|; p < 0 for phi < 0 allows cancellation),
// in FP64 from the exact stored values otherwise.
// clear_fp32: 1 clear, 0 not clear, -1 when only the exact values can tell.
__device__ __forceinline__ int clear_fp32(float phd, float phl) {
  const float fa = p32(phd), fb = p32(phl);
  const float q = fa + fb, err = 1e-6f * (fabsf(fa) + fabsf(fb)) + 1e-20f;
  if (q - err > 1e-10f) return 0;
  if (q + err < 1e-10f) return 1;
  return -1;
}

// the test on the exact values (the reference takes max(phi_pre, sum),
// which skips a NaN sum)
__device__ __forceinline__ bool clear_exact(double phd, double phl) {
  return !(p64(phd) + p64(phl) >= 1e-10);
}

template <class T>
__device__ __forceinline__ bool clear_at(const NucArgs& a, size_t s) {
  const int c = clear_fp32(ldphi_f<T>(a, 2, s), ldphi_f<T>(a, 3, s));
  if (c >= 0) return c == 1;
  return clear_exact(ldval<T>(a, 2, s), ldval<T>(a, 3, s));
}

// Philox draw of a cell in a call: counter (cell, call), key = seed
__device__ __forceinline__ uint4 nuc_draw(const NucArgs& a, long long idx) {
  const unsigned long long call = *a.call_ptr;
  return philox4x32_10(make_uint4(uint32_t(idx), uint32_t(uint64_t(idx) >> 32), uint32_t(call),
                                  uint32_t(call >> 32)),
                       make_uint2(uint32_t(a.seed), uint32_t(a.seed >> 32)));
}

// The FP64 decision of one clear cell (reference linear index idx, storage
// index s) with its draw w: classical nucleation probability of each phase
// against the draw; fills e and returns true on an event.
template <class T>
__device__ __noinline__ bool decide64(const NucArgs& a, long long idx, size_t s, uint4 w, NucEvent& e) {
  const double X = ldval<T>(a, 0, s), Y = ldval<T>(a, 1, s);
  const double u[2] = {u53(w.x, w.y), u53(w.z, w.w)};
  const double dG = g64<0>(X, Y);
  double dcc, dnn;
  diffusivities(X, Y, dcc, dnn);
  int mask = 0;
  double rp[2] = {0.0, 0.0};
#pragma unroll
  for (int ph = 0; ph < 2; ph++) {
    double Rstar = 0.0, P = 0.0;
    probability_sphere(X, Y, dG, dcc, dnn, a.sigma[ph], a.Vatom, a.n_gam, a.dV, a.dt, Rstar, P);
    if (Rstar > 0.) {
      rp[ph] = Rstar / a.dx;
      if (P - u[ph] > 0) {
        if (rp[ph] <= kNucMaxRadius)
          mask |= 1 << ph;
        else
          atomicExch(a.status, 2);  // nucleus wider than the paint limit: reported
      }
    }
  }
  if (!mask) return false;
  e.cell = idx;
  e.mask = mask;
  e.pad = 0;
  e.xcr = X;
  e.xnb = Y;
  e.r[0] = rp[0];
  e.r[1] = rp[1];
  return true;
}

// warp-aggregated append of the lanes' events (whole warp)
__device__ __forceinline__ void append_events(const NucArgs& a, bool ev, const NucEvent& e) {
  const unsigned bal = __ballot_sync(0xffffffffu, ev);
  if (bal == 0) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(bal) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(a.count, unsigned(__popc(bal)));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (ev) {
    const unsigned slot = base + __popc(bal & ((1u << lane) - 1u));
    if (slot < unsigned(a.cap)) a.events[slot] = e;
  }
}


// The FP32 screen of a clear cell whose stored x_Cr, x_Nb round to X, Y (in
// FP32) and whose reference linear index is idx.  Screens on the bound z_up
// of z = dt dV (J_Cr + J_Nb), which carries several nats of analytic slack;
// kNucMargin covers the FP32 evaluation error many times over:
//  * z < 2^-55: FP64 exp(-z) is 1 or 1 - 2^-53, so P_nuc <= 2^-53 <= u for
//    every draw -- no event, no draw needed;
//  * else draw (w), and leave the cell to the FP64 decision unless u >= hi32
//    2^-32 (rounded toward zero) >= P_up >= P_nuc for both phases.
// Returns true when the FP64 decision is needed.  The first tier settles
// about 70 % of the warps of the enriched-stripe workloads; the second tier
// and the draw are inlined for the rest (a call passed its arguments through
// the stack, which cost more than the registers inlining adds).
__device__ __forceinline__ bool nuc_screen_rest(const NucArgs& a, float X, float Y, long long idx,
                                             const ZPre p, float lnz0, float lnz1, uint4* wout) {
  float lnz[2] = {lnz0, lnz1};
  if (p.ok) ln_z_tier2(X, Y, p, a, lnz);
  if (fmaxf(lnz[0], lnz[1]) + kNucMargin < kNucNoDraw) return false;
  const uint4 w = nuc_draw(a, idx);
  *wout = w;
  const float ulo[2] = {__uint2float_rz(w.x) * 0x1p-32f, __uint2float_rz(w.z) * 0x1p-32f};
  bool need = false;
#pragma unroll
  for (int ph = 0; ph < 2; ph++) {
    const bool bounded = lnz[ph] + kNucMargin < 80.0f;
    const float pup = 2.0f * __expf(fminf(lnz[ph] + kNucMargin, 80.0f)) + 0x1p-52f;
    if (!bounded || !(ulo[ph] >= pup)) need = true;
  }
  return need;
}

__device__ __forceinline__ bool nuc_screen(const NucArgs& a, float X, float Y, long long idx,
                                           uint4& w) {
  const ZPre p = z_pre(X, Y);
  float lnz[2];
  ln_z_tier1(p, a, lnz);
  if (fmaxf(lnz[0], lnz[1]) + kNucMargin < kNucNoDraw) return false;
  return nuc_screen_rest(a, X, Y, idx, p, lnz[0], lnz[1], &w);
}

// Cells the screen cannot settle go to k_nuc_fp64 as a compact list: a warp
// issues the FP64 path if any of its lanes needs it, so in place a few such
// cells would cost whole warps.  Cells past the list's capacity decide here,
// from the stored values at storage index s.  Whole warp.
template <class T>
__device__ __forceinline__ void nuc_list_or_decide(const NucArgs& a, bool need, long long idx,
                                                   size_t s, uint4 w) {
  const int lane = threadIdx.x & 31;
  const unsigned nb = __ballot_sync(0xffffffffu, need);
  if (nb == 0) return;
  {
    const int leader = __ffs(nb) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(a.count + 1, unsigned(__popc(nb)));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (need) {
      const unsigned slot = base + __popc(nb & ((1u << lane) - 1u));
      if (slot < unsigned(a.cand_cap)) {
        a.cand[slot] = idx;
        need = false;
      }
    }
  }
  bool ev = false;
  NucEvent e;
  if (need) ev = decide64<T>(a, idx, s, w, e);
  append_events(a, ev, e);
}

}  // namespace
}  // namespace pfa
