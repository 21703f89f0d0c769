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
#include "pfa_nucleation.h"

namespace pfa {

using namespace dev;

namespace {

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

// Upper bound, in FP32, of ln z with z = dt dV (J_Cr + J_Nb) for each phase;
// +inf where no bound is attempted (compositions outside the simplex, or
// above the gamma equilibrium composition, where the exponents change sign).
// The diffusivities are bounded by the magnitudes of their three mobility
// terms, so the bound holds whatever the signs of D_CrCr and D_NbNb:
//   |D| <= 3 x 1.5e-20 x exp(max e) x 2.5e6     (prefactors, |s| + add)
//   k1  <= 3 G* |D| / (sigma a^4) x Zeldovich x n_gam      (x <= 1)
//   J_Cr + J_Nb <= 2 k1 exp(-k2 / max(dc_Cr, dc_Nb)),  k2 = G* / kT.
// With G* = 16 pi sigma^3 / (3 dG^2) and Zeldovich ~ dG^2 the dG factors of
// k1 cancel, so ln z <= lnC1 + max e - C2 / (dG^2 max dc) with the per-phase
// constants lnC1, C2 of the host (NucArgs).
__device__ void ln_z_bound(float X, float Y, const NucArgs& a, float lnz[2]) {
  lnz[0] = lnz[1] = INFINITY;
  const float dcCr = float(kXe[0][0]) - X, dcNb = Y - float(kXe[0][1]);
  if (!(dcCr > 0.0f && dcNb > 0.0f && X > 0.0f && Y > 0.0f && X + Y < 1.0f)) return;
  const float u = X - float(kXe[0][0]), v = Y - float(kXe[0][1]);
  const float dG = float(kG[0][0]) * u * u + (float(kG[0][1]) * X - float(kG[0][2])) * v +
                   float(kG[0][3]) * v * v;
  if (!(dG > 1.0f)) return;
  const float xni = 1.0f - X - Y;
  const float eNb = -34.982563536715503f * Y * xni + 14.437947842988088f * Y;
  const float eCr = -7.1543718172640256f * X * xni + 3.3541967644499233f * X;
  const float eNi = -8.5221193705645018f * X * xni + 4.0036674816806448f * X -
                    442.62877981749585f * Y * xni - 0.82164267100913768f * Y;
  const float emax = fmaxf(eNb, fmaxf(eCr, eNi));
  const float inv = __fdividef(1.0f, dG * dG * fmaxf(dcCr, dcNb));
#pragma unroll
  for (int ph = 0; ph < 2; ph++) {
    const float l = a.lnC1[ph] + emax - a.C2[ph] * inv;
    if (l == l) lnz[ph] = l;  // NaN stays +inf
  }
}

// p(phi_del) + p(phi_lav) < 1e-10 as the reference's FP64 test decides it:
// in FP32 when the FP32 sum is farther from the threshold than its error
// bound (1e-6 of |p_del| + |p_lav|; p < 0 for phi < 0 allows cancellation),
// in FP64 from the exact stored values otherwise.
template <class T>
__device__ __forceinline__ bool clear_at(const NucArgs& a, size_t s) {
  const float fa = p32(ldphi_f<T>(a, 2, s)), fb = p32(ldphi_f<T>(a, 3, s));
  const float q = fa + fb, err = 1e-6f * (fabsf(fa) + fabsf(fb)) + 1e-20f;
  if (q - err > 1e-10f) return false;
  if (q + err < 1e-10f) return true;
  // the reference takes max(phi_pre, sum), which skips a NaN sum
  return !(p64(ldval<T>(a, 2, s)) + p64(ldval<T>(a, 3, s)) >= 1e-10);
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
__device__ bool decide64(const NucArgs& a, long long idx, size_t s, uint4 w, NucEvent& e) {
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

template <class T>
__global__ void __launch_bounds__(256) k_nuc_decide(NucArgs a) {
  const int gx = blockIdx.x * 32 + (threadIdx.x & 31);
  const int gy = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
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
      const T Xs = static_cast<const T*>(a.f[0])[s * a.stride];
      const T Ys = static_cast<const T*>(a.f[1])[s * a.stride];
      // Screen in FP32 on the bound z_up of z = dt dV (J_Cr + J_Nb), which
      // carries several nats of analytic slack; kMargin covers the FP32
      // evaluation error many times over:
      //  * z < 2^-55: FP64 exp(-z) is 1 or 1 - 2^-53, so P_nuc <= 2^-53 <= u for
      //    every draw -- no event, no draw needed;
      //  * else draw, and skip the FP64 path when u >= hi32 2^-32 (rounded
      //    toward zero) >= P_up >= P_nuc.
      constexpr float kMargin = 2.0f;
      float lnz[2];
      ln_z_bound(float(Xs), float(Ys), a, lnz);
      const float lnz_max = fmaxf(lnz[0], lnz[1]) + kMargin;
      if (!(lnz_max < -38.8f)) {  // ln 2^-56
        w = nuc_draw(a, idx);
        const float ulo[2] = {__uint2float_rz(w.x) * 0x1p-32f, __uint2float_rz(w.z) * 0x1p-32f};
#pragma unroll
        for (int ph = 0; ph < 2; ph++) {
          const bool bounded = lnz[ph] + kMargin < 80.0f;
          const float pup = 2.0f * __expf(fminf(lnz[ph] + kMargin, 80.0f)) + 0x1p-52f;
          if (!bounded || !(ulo[ph] >= pup)) need = true;
        }
      }
    }
  }
  // Cells the screen cannot settle go to k_nuc_fp64 as a compact list: a warp
  // issues the FP64 path if any of its lanes needs it, so in place a few such
  // cells would cost whole warps.  Cells past the list's capacity decide here.
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

// The FP64 decisions of the listed cells, 32 per warp.
template <class T>
__global__ void __launch_bounds__(256) k_nuc_fp64(NucArgs a) {
  const unsigned n = min(a.count[1], unsigned(a.cand_cap));
  const int lane = threadIdx.x & 31;
  const unsigned step = gridDim.x * blockDim.x;  // a multiple of 32: warps stay whole
  const long long nxr = a.Nx + 2, nyr = a.Ny + 2;
  for (unsigned b = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); b < n; b += step) {
    const unsigned i = b + lane;
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

template <class T>
__global__ void __launch_bounds__(1024) k_nuc_apply(NucArgs a) {
  extern __shared__ unsigned long long s_key[];
  const unsigned n = *a.count;
  __syncthreads();
  // the decision kernel of this call has read the counter: advance it
  if (threadIdx.x == 0) *a.call_ptr += 1ull;
  if (n == 0) return;
  if (n > unsigned(a.cap)) {
    if (threadIdx.x == 0) *a.status = 1;  // overflow: nothing painted
    return;
  }
  unsigned m = 1;
  while (m < n) m <<= 1;
  for (unsigned t = threadIdx.x; t < m; t += blockDim.x)
    s_key[t] = t < n ? ((unsigned long long)a.events[t].cell << kNucIdxBits) | t : ~0ull;
  __syncthreads();
  // bitonic sort, ascending
  for (unsigned k = 2; k <= m; k <<= 1)
    for (unsigned j = k >> 1; j > 0; j >>= 1) {
      for (unsigned t = threadIdx.x; t < m; t += blockDim.x) {
        const unsigned p = t ^ j;
        if (p > t) {
          const unsigned long long u = s_key[t], v = s_key[p];
          const bool up = (t & k) == 0;
          if ((u > v) == up) {
            s_key[t] = v;
            s_key[p] = u;
          }
        }
      }
      __syncthreads();
    }
  for (unsigned q = 0; q < n; q++) {
    const NucEvent e = a.events[s_key[q] & ((1ull << kNucIdxBits) - 1)];
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
  const size_t smem = sizeof(unsigned long long) * size_t(kNucCap);
  const int fp64_blocks = 152 * 4;  // grid-stride over the list (its length is on the device)
  if (a.is_f32) {
    k_nuc_decide<float><<<grid, 256, 0, s>>>(a);
    k_nuc_fp64<float><<<fp64_blocks, 256, 0, s>>>(a);
    k_nuc_apply<float><<<1, 1024, smem, s>>>(a);
  } else {
    k_nuc_decide<double><<<grid, 256, 0, s>>>(a);
    k_nuc_fp64<double><<<fp64_blocks, 256, 0, s>>>(a);
    k_nuc_apply<double><<<1, 1024, smem, s>>>(a);
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
  // constants of the FP32 screening bound (ln_z_bound):
  // ln z <= lnC1 + max e - C2 / (dG^2 max dc)
  for (int ph = 0; ph < 2; ph++) {
    const double sg = a.sigma[ph], s3 = sg * sg * sg;
    const double a4 = std::pow(kLatticeConst, 4);
    const double lnDpre = std::log(3.0 * 1.5e-20 * 2.5e6);            // |D| prefactor bound
    const double lnG = std::log(16.0 * kPi * s3 / 3.0);                  // G* dG^2
    const double lnZ = std::log(a.Vatom / (8.0 * kPi * std::sqrt(kKT * s3)));  // Zeldovich / dG^2
    a.lnC1[ph] = float(std::log(3.0) + lnG - std::log(sg) - std::log(a4) + lnDpre + lnZ +
                       a.ln_ngam + std::log(2.0) + a.ln_dtdV);
    a.C2[ph] = float(16.0 * kPi * s3 / (3.0 * kKT));
  }
  return nullptr;
}

cudaError_t nucleation_setup() {
  const int smem = int(sizeof(unsigned long long) * kNucCap);
  cudaError_t e = cudaFuncSetAttribute(k_nuc_apply<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_nuc_apply<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

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
