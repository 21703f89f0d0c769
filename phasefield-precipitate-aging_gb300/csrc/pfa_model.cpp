// pfa_model.cpp -- host-side model parameters of libpfa_gb300.
//
// Computes what the reference's host code computes before the loop
// (src/main.cpp:252-268): the constant diffusion matrix
// (set_diffusion_matrix, src/alloy625.cpp:80-109), kappa and omega
// (src/parameters.h:42-48), the Allen-Cahn mobility and the time step, plus
// the derived coefficients of the FP32 fast path.
#include <cmath>
#include <cstring>

#include "pfa_internal.h"
#include "pfa_model.h"

namespace pfa {

namespace {

double mob(int k, double X, double Y) {
  // Redlich-Kister mobility exponents of thermo/parabola625.c:1860-1894
  const double xni = -X - Y + 1;
  if (k == 0) return kMobPreNb * std::exp(-34.982563536715503 * Y * xni + 14.437947842988088 * Y);
  if (k == 1) return kMobPreCr * std::exp(-7.1543718172640256 * X * xni + 3.3541967644499233 * X);
  return kMobPreNi * std::exp(-8.5221193705645018 * X * xni + 4.0036674816806448 * X -
                              442.62877981749585 * Y * xni - 0.82164267100913768 * Y);
}

}  // namespace

double model_D(int row, int col, double X, double Y) {
  const double xni = -X - Y + 1;
  const double mNb = mob(0, X, Y), mCr = mob(1, X, Y), mNi = mob(2, X, Y);
  const double s = col == 0 ? (-kHCrCr * X - kHCrNb * Y) : (-kHCrNb * X - kHNbNb * Y);
  const double add_cr = col == 0 ? kHCrCrAdd : kHCrNbAddB;
  const double add_nb = col == 0 ? kHCrNbAddA : kHNbNbAdd;
  if (row == 0)
    return -mNb * X * Y * (s + add_nb) + mCr * X * (1 - X) * (s + add_cr) - mNi * X * s * xni;
  return -mCr * X * Y * (s + add_cr) + mNb * Y * (1 - Y) * (s + add_nb) - mNi * Y * s * xni;
}

// Spectral radius of D * (d x^gamma / d X) over the phase simplex.  x^gamma
// is linear in X, so the Jacobian is the X-block of the gamma numerators over
// the shared denominator.
double model_kks_diffusivity(const double Dcr[2], const double Dnb[2]) {
  double worst = 0.0;
  const int n = 100;
  for (int a = 0; a <= n; a++)
    for (int b = 0; a + b <= n; b++) {
      const double pd = double(a) / n, pl = double(b) / n, pg = 1.0 - pd - pl;
      const double lin[3] = {pd, pg, pl};
      const double mono[6] = {pd * pd, pd * pg, pd * pl, pg * pg, pg * pl, pl * pl};
      double den = 0.0;
      for (int k = 0; k < 6; k++) den += kDen[k] * mono[k];
      double J[2][2];
      for (int i = 0; i < 2; i++) {
        double lc = 0.0, lm = 0.0;
        for (int k = 0; k < 3; k++) {
          lc += kFict[0][i].l[k] * lin[k];
          lm += kFict[0][i].m[k] * lin[k];
        }
        J[i][0] = kFict[0][i].scale * lc / den;
        J[i][1] = kFict[0][i].scale * lm / den;
      }
      const double m00 = Dcr[0] * J[0][0] + Dcr[1] * J[1][0];
      const double m01 = Dcr[0] * J[0][1] + Dcr[1] * J[1][1];
      const double m10 = Dnb[0] * J[0][0] + Dnb[1] * J[1][0];
      const double m11 = Dnb[0] * J[0][1] + Dnb[1] * J[1][1];
      const double tr = m00 + m11, det = m00 * m11 - m01 * m10;
      const double disc = 0.25 * tr * tr - det;
      double rho;
      if (disc >= 0.0) {
        const double s = std::sqrt(disc);
        rho = std::fmax(std::fabs(0.5 * tr + s), std::fabs(0.5 * tr - s));
      } else {
        rho = std::sqrt(det);
      }
      worst = std::fmax(worst, rho);
    }
  return worst;
}

void model_fast_coef(FastCoef* o) {
  std::memset(o, 0, sizeof(*o));
  for (int k = 0; k < 6; k++) o->den[k] = float(kDen[k]);
  for (int c = 0; c < 2; c++) {
    const FictRow& r = kFict[0][c];
    for (int k = 0; k < 3; k++) {
      o->num[c][k] = float(r.scale * r.l[k]);
      o->num[c][3 + k] = float(r.scale * r.m[k]);
    }
    for (int k = 0; k < 6; k++) o->num[c][6 + k] = float(r.scale * r.q[k]);
  }
  // Grand-potential difference Delta P_i(u), u = x^gamma - xe_gamma.  With
  // g = 1/2 u^T H u + e u_2 (e = B xeCr - C) and equal chemical potentials,
  //   Delta P = u^T [1/2 (Hg S Hg - Hg)] u + [f (S Hg)_2 - Hg dxe] . u
  //             + 1/2 f^2 S_22 - e_g dxe_2,
  // S = H_i^-1, f = e_g - e_i, dxe = xe_gamma - xe_i.
  auto H = [](int ph, double h[2][2]) {
    h[0][0] = 2 * kG[ph][0];
    h[0][1] = h[1][0] = kG[ph][1];
    h[1][1] = 2 * kG[ph][3];
  };
  auto e_of = [](int ph) { return kG[ph][1] * kXe[ph][0] - kG[ph][2]; };
  double Hg[2][2];
  H(0, Hg);
  const double eg = e_of(0);
  for (int ph = 1; ph <= 2; ph++) {
    double Hi[2][2];
    H(ph, Hi);
    const double det = Hi[0][0] * Hi[1][1] - Hi[0][1] * Hi[1][0];
    const double S[2][2] = {{Hi[1][1] / det, -Hi[0][1] / det}, {-Hi[1][0] / det, Hi[0][0] / det}};
    const double f = eg - e_of(ph);
    const double dxe[2] = {kXe[0][0] - kXe[ph][0], kXe[0][1] - kXe[ph][1]};
    double SH[2][2], HSH[2][2];
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) SH[i][j] = S[i][0] * Hg[0][j] + S[i][1] * Hg[1][j];
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) HSH[i][j] = Hg[i][0] * SH[0][j] + Hg[i][1] * SH[1][j];
    double Q[2][2];
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) Q[i][j] = 0.5 * (HSH[i][j] - Hg[i][j]);
    const double l0 = f * SH[1][0] - (Hg[0][0] * dxe[0] + Hg[0][1] * dxe[1]);
    const double l1 = f * SH[1][1] - (Hg[1][0] * dxe[0] + Hg[1][1] * dxe[1]);
    const double c0 = 0.5 * f * f * S[1][1] - eg * dxe[1];
    float* out = o->dP[ph - 1];
    out[0] = float(c0);
    out[1] = float(l0);
    out[2] = float(l1);
    out[3] = float(Q[0][0]);
    out[4] = float(Q[0][1] + Q[1][0]);
    out[5] = float(Q[1][1]);
  }
  o->xe_gam[0] = float(kXe[0][0]);
  o->xe_gam[1] = float(kXe[0][1]);
  for (int ph = 0; ph < 3; ph++)
    for (int c = 0; c < 2; c++) {
      o->xe_hi[ph][c] = float(kXe[ph][c]);
      o->xe_lo[ph][c] = float(kXe[ph][c] - double(o->xe_hi[ph][c]));
    }
  // equilibrium-referenced form (FastCoef::dev): quadratic coefficients of
  // l . [pD pG pL] on the monomials pD^2, pD pG, pD pL, pG^2, pG pL, pL^2
  auto homog = [](const double l[3], double q[6]) {
    q[0] = l[0];
    q[1] = l[0] + l[1];
    q[2] = l[0] + l[2];
    q[3] = l[1];
    q[4] = l[1] + l[2];
    q[5] = l[2];
  };
  static const int kMono[5] = {0, 1, 2, 4, 5};  // all but pG^2
  for (int c = 0; c < 2; c++) {
    const FictRow& r = kFict[0][c];
    double lx[3], ly[3], qx[6], qy[6];
    for (int k = 0; k < 3; k++) {
      lx[k] = r.scale * r.l[k];
      ly[k] = r.scale * r.m[k];
    }
    homog(lx, qx);
    homog(ly, qy);
    for (int j = 0; j < 6; j++) (c == 0 ? qx : qy)[j] -= kDen[j];  // - X_c den
    for (int t = 0; t < 5; t++) {
      const int j = kMono[t];
      o->dev[c][t][0] = float(qx[j]);
      o->dev[c][t][1] = float(qy[j]);
    }
  }
}

}  // namespace pfa
