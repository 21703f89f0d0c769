// pfa_internal.h -- shared declarations of libpfa_gb300 (not installed).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace pfa {

// Per-grid model constants (double on the host; the FP32 kernels round them).
struct ModelConst {
  double D[2][2];    // D[0] = [D_CrCr, D_CrNb], D[1] = [D_NbCr, D_NbNb]
  double kappa[2];   // gradient coefficients (delta, laves)
  double omega[2];   // well heights
  double L[2];       // Allen-Cahn mobilities
  double alpha;      // three-phase penalty
  double dt;         // time step
  double mask[5];    // 5-point mask: north, west, centre, east, south (2D)
  double idx2[3];    // 1/dx^2, 1/dy^2, 1/dz^2
};

// Coefficients of the FP32 fast path, derived on the host in double.
//  * gamma solve in the reference's three-variable form (all denominator
//    terms are non-negative on the simplex, so it does not cancel):
//      den   = d . [pD^2, pD pG, pD pL, pG^2, pG pL, pL^2]
//      num_k = XCR (l_k . [pD pG pL]) + XNB (m_k . [pD pG pL]) + q_k . monomials
//    with the scale folded into l, m, q;  x^gamma_k = num_k / den.
//  * grand-potential difference of phase i as a quadratic in
//      u = x^gamma - xe_gamma:  c0 + u1 (c1 + c11 u1 + c12 u2) + u2 (c2 + c22 u2)
//  * equilibrium-referenced form of the same solve.  The system is linear in
//    X, and the mixture X*(p) = sum_i p_i xe_i of the phases' equilibrium
//    compositions (a common tangent of the paraboloids) gives x^gamma =
//    xe_gamma for every p.  Hence, with d = X - X*(p),
//      u = x^gamma - xe_gamma = d + (A(p) d_Cr + B(p) d_Nb) / den,
//    A_k, B_k = sums over the monomials that contain pD or pL (pD^2, pD pG,
//    pD pL, pG pL, pL^2) of the quadratic forms of (l_k - den e_k) and m_k
//    (linear terms written as quadratics with pD + pG + pL = 1; the pG^2
//    coefficients vanish).  Inside a precipitate d is small even where the
//    KKS amplification A/den is large, so FP32 keeps u accurate; the plain
//    num / den form loses it to cancellation in num.
struct FastCoef {
  float den[6];        // d
  float num[2][12];    // per comp: l0 l1 l2 m0 m1 m2 q0..q5
  float dP[2][6];      // per phase (delta, laves): c0 c1 c2 c11 c12 c22
  float xe_gam[2];     // xe_gamma rounded to FP32
  float dev[2][5][2];  // per comp, per monomial (pD^2 pD pG pD pL pG pL pL^2): A B
  float xe_hi[3][2];   // equilibrium compositions (gamma, delta, laves), FP32 part
  float xe_lo[3][2];   // and their remainders
};

void model_fast_coef(FastCoef* out);

// The FP32 form's kernels index a grid's (2D) or a plane's (3D) records with
// 32-bit integers: rows of ceil(Nx / 32) * 32 records, Ny rows, below 2^31.
inline bool fp32_records_fit(int Nx, int Ny) {
  return (long long)((Nx + 31) / 32) * 32 * Ny < (1LL << 31);
}

// Host model helpers (pfa_model.cpp)
double model_D(int row, int col, double xcr, double xnb);
double model_kks_diffusivity(const double Dcr[2], const double Dnb[2]);

// Sticky error word of the library (last failure); see pfa_gb300.h.
void set_error(int code, const char* where);

}  // namespace pfa
