/*
 * pfa_oracle.c -- CPU oracle: restated model energies + step semantics.
 *
 * TEST INFRASTRUCTURE ONLY (see pfa_oracle.h).  Loaded by the tests, the
 * smoke check and the benchmark's CPU-baseline leg; never by the product.
 *
 * The energy constants below are the model data baked into the reference's
 * generated thermo/parabola625.c; the functions are written here as
 * coefficient tables evaluated by small loops.  tests/golden holds vectors
 * made by the reference's own compiled functions, which pin these tables.
 */
#include <math.h>
#include <stdint.h>
#include "pfa_oracle.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---- constants: thermo/parabola625.c:38-117 (kT, RT, Vm, xe_*) ---- */
static const double K_T = 1.5782889043500002e-20;
static const double R_T = 9504.6840941999999;
static const double V_M = 1.0000000000000001e-5;
static const double SIGMA_DEFAULT = 0.13;           /* s_delta, s_laves: :299-315 */
static const double LATTICE_CONST = 0.352e-9;       /* src/parameters.h:26 */

/* equilibrium compositions [gam, del, lav][Cr, Nb], thermo/parabola625.c:65-117 */
static const double XE[3][2] = {
	{0.52421634830562147, 0.01299272922003303},
	{0.022966218927631978, 0.24984563695705883},
	{0.37392129441013022, 0.25826261799015571},
};

/* Paraboloids g = A (XCR - xeCr)^2 + (B XCR - C)(XNB - xeNb) + E (XNB - xeNb)^2,
 * thermo/parabola625.c:418-443.  Columns: A, B, C, E. */
static const double GPAR[3][4] = {
	{2267132212.7620249, 15095482346.486225, 7913298631.5869827, 55193083240.685936},
	{21346492990.798885, 16906497386.287418, 388278320.27291465, 3085369132931.8848},
	{8866730284.8069954, 24191004361.532181, 9045531663.945219, 98294310279.883911},
};

/* gamma chemical potentials, thermo/parabola625.c:655-671: a*XCR + b*XNB + c */
static const double DGGAM[2][3] = {
	{4534264425.5240498, 15095482346.486225, -2573067053.9739881},
	{15095482346.486225, 110386166481.37187, -9347516202.3169327},
};

/* Fictitious compositions, thermo/parabola625.c:245-297.  Each is
 *   scale * ( XCR*(l0 pDel + l1 pGam + l2 pLav) + XNB*(m0 pDel + m1 pGam + m2 pLav)
 *            + q . [pDel^2, pDel pGam, pDel pLav, pGam^2, pGam pLav, pLav^2] ) / den
 * with the shared denominator den = d . [same six monomials]. */
static const double FDEN[6] = {
	0.001036042775998007, 0.12229015747171917, 0.041785936156220213,
	1.0, 0.73028945399293654, 0.093983883345629876,
};
typedef struct {
	double scale;
	double l[3], m[3];
	double q[6];
} fict_row;
static const fict_row FICT[3][2] = {
	{ /* gamma */
		{1.0, {0.016938286205500769, 1.0, 0.54889980006097594},
		 {-0.3468746660495467, 0.0, -0.10246420218061991},
		 {0.086819224054883945, 0.036767802923980249, 0.11815012520929236,
		  0.0, -0.27750258277182049, -0.12951476250779617}},
		{-1.0, {0.0021576593653206376, 0.0, 0.054466450838266962},
		 {-0.10535187126621841, -1.0, -0.18138965393196074},
		 {0.026258691080522339, 0.24849448207756414, 0.06992726713680375,
		  0.0, 0.22257870755542869, 0.025258893954068839}},
	},
	{ /* delta */
		{0.3468746660495467, {0.0029867928603642137, 0.30371739875396442, 0.11224396861282376},
		 {0.0, 1.0, 0.15026949298026254},
		 {0.0, -0.25028989589710454, -0.038472217853981416,
		  -0.10599737173866837, -0.38426983287411109, -0.074556825343604527}},
		{0.24849448207756414, {0.0, 0.0086829266681549659, 0.0010534256500958396},
		 {0.0041692787998190662, 0.068163631095090937, 0.011474488301439056},
		 {0.0, 0.10567112340275649, 0.038045328588644858,
		  1.0, 0.71270814650507497, 0.091137578230976013}},
	},
	{ /* laves */
		{0.27750258277182055, {0.010275028791049912, 0.65365032685519298, 0.33867750853659306},
		 {-0.18783493715380425, 0.36923693162478488, 0.0},
		 {0.04808977843373196, 0.054570103782716275, 0.093195074562756067,
		  1.0, 0.46671552103819908, 0.0}},
		{-0.54889980006097605, {0.00047690026722310247, -0.099228403494073802, 0.0},
		 {-0.070932051941581864, -1.0, -0.1712222947342838},
		 {0.017223643043877624, 0.19525744879034301, 0.041259234012827196,
		  -0.40549970601319757, -0.046017313089315913, 0.0}},
	},
};

/* Diffusivities, thermo/parabola625.c:1860-1894.  Three atomic-mobility
 * prefactors with Redlich-Kister exponents, M_k = pre_k exp(e_k), and the
 * second-derivative weights h of the gamma paraboloid (divided by RT). */
static const double MOB_PRE_NB = 1.4170990277916469e-20;
static const double MOB_PRE_CR = 3.5027570743586952e-21;
static const double MOB_PRE_NI = 1.8295676400933012e-21;
static const double H_CRCR = 45342.644255240499;
static const double H_CRNB = 150954.82346486227;
static const double H_NBNB = 1103861.6648137188;
/* the additive copies of the same weights carry their own last digits */
static const double H_CRNB_ADD_A = 150954.82346486227;  /* D_CrCr, D_NbCr */
static const double H_CRNB_ADD_B = 150954.82346486225;  /* D_CrNb, D_NbNb */
static const double H_NBNB_ADD = 1103861.664813719;
static const double H_CRCR_ADD = 45342.644255240499;

static double mob_nb(double XCR, double XNB)
{
	return exp(-34.982563536715503 * XNB * (-XCR - XNB + 1) + 14.437947842988088 * XNB);
}
static double mob_cr(double XCR, double XNB)
{
	return exp(-7.1543718172640256 * XCR * (-XCR - XNB + 1) + 3.3541967644499233 * XCR);
}
static double mob_ni(double XCR, double XNB)
{
	return exp(-8.5221193705645018 * XCR * (-XCR - XNB + 1) + 4.0036674816806448 * XCR
	           - 442.62877981749585 * XNB * (-XCR - XNB + 1) - 0.82164267100913768 * XNB);
}

double orc_kT(void) { return K_T; }
double orc_RT(void) { return R_T; }
double orc_Vm(void) { return V_M; }
double orc_xe(int phase, int comp) { return XE[phase][comp]; }

/* p(x) = x^3 (6x^2 - 15x + 10), thermo/parabola625.c:11-18 */
double orc_p(double x)
{
	return pow(x, 3) * (6.0 * pow(x, 2) - 15.0 * x + 10.0);
}

/* p'(x) = 30 x^2 (1 - x)^2, thermo/parabola625.c:20-27 */
double orc_pprime(double x)
{
	return 30.0 * pow(x, 2) * pow(1.0 - x, 2);
}

double orc_fict(int phase, int comp, double xcr, double xnb,
                double pdel, double pgam, double plav)
{
	const fict_row* r = &FICT[phase][comp];
	const double lin[3] = {pdel, pgam, plav};
	const double mono[6] = {pdel * pdel, pdel * pgam, pdel * plav,
	                        pgam * pgam, pgam * plav, plav * plav};
	double num = 0.0, den = 0.0;
	for (int k = 0; k < 3; k++)
		num += xcr * r->l[k] * lin[k] + xnb * r->m[k] * lin[k];
	for (int k = 0; k < 6; k++) {
		num += r->q[k] * mono[k];
		den += FDEN[k] * mono[k];
	}
	return r->scale * num / den;
}

double orc_g(int phase, double xcr, double xnb)
{
	const double* g = GPAR[phase];
	const double ucr = xcr - XE[phase][0];
	const double unb = xnb - XE[phase][1];
	return g[0] * ucr * ucr + (g[1] * xcr - g[2]) * unb + g[3] * unb * unb;
}

double orc_dg_gam(int comp, double xcr, double xnb)
{
	return DGGAM[comp][0] * xcr + DGGAM[comp][1] * xnb + DGGAM[comp][2];
}

/* d g_<phase> / d x_<comp> and the (constant) curvatures d2 g / dx_i dx_j of
 * the paraboloids (thermo/parabola625.c:655-706, 1305-1410), derived here
 * from the energy parameters above: with u = XCR - xe_Cr, v = XNB - xe_Nb,
 *   g = A u^2 + (B XCR - C) v + E v^2,
 *   dg/dXCR = 2 A u + B v,  dg/dXNB = B XCR - C + 2 E v,
 *   d2g = [[2 A, B], [B, 2 E]]. */
double orc_dg(int phase, int comp, double xcr, double xnb)
{
	const double* g = GPAR[phase];
	const double ucr = xcr - XE[phase][0];
	const double unb = xnb - XE[phase][1];
	if (comp == 0)
		return 2.0 * g[0] * ucr + g[1] * unb;
	return g[1] * xcr - g[2] + 2.0 * g[3] * unb;
}

double orc_d2g(int phase, int i, int j)
{
	const double* g = GPAR[phase];
	if (i != j)
		return g[1];
	return i == 0 ? 2.0 * g[0] : 2.0 * g[3];
}

/* D[row][col]: row 0 = Cr, 1 = Nb; col 0 = Cr, 1 = Nb. */
double orc_D(int row, int col, double XCR, double XNB)
{
	const double xNi = -XCR - XNB + 1;
	const double mNb = MOB_PRE_NB * mob_nb(XCR, XNB);
	const double mCr = MOB_PRE_CR * mob_cr(XCR, XNB);
	const double mNi = MOB_PRE_NI * mob_ni(XCR, XNB);
	/* s = -(h_col,Cr XCR + h_col,Nb XNB): gradient of the curvature row */
	const double s = (col == 0) ? (-H_CRCR * XCR - H_CRNB * XNB) : (-H_CRNB * XCR - H_NBNB * XNB);
	const double add_cr = (col == 0) ? H_CRCR_ADD : H_CRNB_ADD_B;
	const double add_nb = (col == 0) ? H_CRNB_ADD_A : H_NBNB_ADD;
	if (row == 0)
		return -mNb * XCR * XNB * (s + add_nb) + mCr * XCR * (1 - XCR) * (s + add_cr)
		       - mNi * XCR * s * xNi;
	return -mCr * XCR * XNB * (s + add_cr) + mNb * XNB * (1 - XNB) * (s + add_nb)
	       - mNi * XNB * s * xNi;
}

/* Classical nucleation theory, thermo/nucleation.c:30-69.  The lattice
 * constant in B* is the compile-time one (src/parameters.h:26), not the
 * Vatom argument. */
void orc_nucleation_probability_sphere(double xCr, double xNb, double dG_chem,
                                       double D_CrCr, double D_NbNb, double sigma,
                                       double Vatom, double n_gam, double dV, double dt,
                                       double* Rstar, double* P_nuc)
{
	const double sigma_cubed = sigma * sigma * sigma;
	const double Zeldov = (Vatom * dG_chem * dG_chem) / (8. * M_PI * sqrt(K_T * sigma_cubed));
	const double Gstar = (16. * M_PI * sigma_cubed) / (3. * dG_chem * dG_chem);
	const double a4 = pow(LATTICE_CONST, 4);
	const double BstarCr = (3. * Gstar * D_CrCr * xCr) / (sigma * a4);
	const double BstarNb = (3. * Gstar * D_NbNb * xNb) / (sigma * a4);
	const double k1Cr = BstarCr * Zeldov * n_gam;
	const double k1Nb = BstarNb * Zeldov * n_gam;
	const double k2 = Gstar / K_T;
	const double dc_Cr = -xCr + XE[0][0];
	const double dc_Nb = xNb - XE[0][1];
	const double JCr = k1Cr * exp(-k2 / dc_Cr);
	const double JNb = k1Nb * exp(-k2 / dc_Nb);
	const double P0 = exp(-dt * dV * (JCr + JNb));
	*P_nuc = 1. - P0;
	*Rstar = (2. * sigma) / dG_chem;
}

/* Spectral radius of D J over the phase simplex, where J = d x^gamma / d X.
 * x^gamma is linear in X (thermo/parabola625.c:245-261), so J is the
 * X-coefficient block of the gamma numerators over the shared denominator.
 * Inside the delta phase J reaches ~100, which makes the effective
 * diffusivity ~58x max(D_CrCr, D_NbNb). */
double orc_kks_diffusivity(const double Dcr[2], const double Dnb[2])
{
	double worst = 0.0;
	const int n = 100;
	for (int a = 0; a <= n; a++)
		for (int b = 0; a + b <= n; b++) {
			const double pd = (double)a / n, pl = (double)b / n, pg = 1.0 - pd - pl;
			const double lin[3] = {pd, pg, pl};
			const double mono[6] = {pd * pd, pd * pg, pd * pl, pg * pg, pg * pl, pl * pl};
			double den = 0.0;
			for (int k = 0; k < 6; k++)
				den += FDEN[k] * mono[k];
			double J[2][2];
			for (int i = 0; i < 2; i++) {
				double lc = 0.0, lm = 0.0;
				for (int k = 0; k < 3; k++) {
					lc += FICT[0][i].l[k] * lin[k];
					lm += FICT[0][i].m[k] * lin[k];
				}
				J[i][0] = FICT[0][i].scale * lc / den;
				J[i][1] = FICT[0][i].scale * lm / den;
			}
			const double m00 = Dcr[0] * J[0][0] + Dcr[1] * J[1][0];
			const double m01 = Dcr[0] * J[0][1] + Dcr[1] * J[1][1];
			const double m10 = Dnb[0] * J[0][0] + Dnb[1] * J[1][0];
			const double m11 = Dnb[0] * J[0][1] + Dnb[1] * J[1][1];
			const double tr = m00 + m11, det = m00 * m11 - m01 * m10;
			const double disc = 0.25 * tr * tr - det;
			double rho;
			if (disc >= 0.0) {
				const double s = sqrt(disc);
				rho = fmax(fabs(0.5 * tr + s), fabs(0.5 * tr - s));
			} else {
				rho = sqrt(det);
			}
			worst = fmax(worst, rho);
		}
	return worst;
}

/* Model parameters as src/main.cpp:252-268 computes them: D from
 * src/alloy625.cpp:80-109 at (xcr0, xnb0), kappa/omega from
 * src/parameters.h:42-48, L from src/alloy625.cpp:102-104.
 * dt_rule 0: the reference's dt, floor(r LinStab min(dt_T, dt_D)) / r with
 *   dt_D = meshres^2 / (4 max(D_CrCr, D_NbNb)) (src/alloy625.cpp:111-121) and
 *   meshres standing for the compile-time spacing (src/parameters.h:18).
 * dt_rule 1: half the explicit stability limit of the KKS system,
 *   min(dt_T, dx^2 / (2 dim rho(D J))), rounded the same way.  The
 *   reference's dt_D ignores the KKS amplification and is unstable inside
 *   delta particles (dt above the limit by 17% at dx = 5 nm). */
void orc_model_params_rule(double dx, double ifce_width, double xcr0, double xnb0,
                           double meshres, int dim, int dt_rule, orc_params* o)
{
	o->D_Cr[0] = orc_D(0, 0, xcr0, xnb0);
	o->D_Cr[1] = orc_D(0, 1, xcr0, xnb0);
	o->D_Nb[0] = orc_D(1, 0, xcr0, xnb0);
	o->D_Nb[1] = orc_D(1, 1, xcr0, xnb0);
	for (int i = 0; i < 2; i++) {
		o->kappa[i] = 3. * SIGMA_DEFAULT * ifce_width / 2.2;
		o->omega[i] = 18. * SIGMA_DEFAULT * SIGMA_DEFAULT / o->kappa[i];
	}
	const double Dnorm = sqrt(o->D_Cr[0] * o->D_Cr[0] + o->D_Nb[1] * o->D_Nb[1]);
	o->Lmob[0] = 1.0 * Dnorm / (ifce_width * ifce_width * R_T / V_M);
	o->Lmob[1] = o->Lmob[0];
	o->alpha = 1.07e11;
	double target;
	if (dt_rule == 0) {
		const double dtT = (meshres * meshres) / (2.0 * dim * o->Lmob[0] * o->kappa[0]);
		const double dtD = (meshres * meshres) / (4.0 * fmax(o->D_Cr[0], o->D_Nb[1]));
		target = 0.02 * fmin(dtT, dtD);
	} else {
		const double dtT = (dx * dx) / (2.0 * dim * o->Lmob[0] * o->kappa[0]);
		const double dtD = (dx * dx) / (2.0 * dim * orc_kks_diffusivity(o->D_Cr, o->D_Nb));
		target = 0.5 * fmin(dtT, dtD);
	}
	double round_dt = 0.0, roundoff = 4e6;
	while (round_dt < 1e-20) {
		roundoff *= 10;
		round_dt = floor(roundoff * target) / roundoff;
	}
	o->dt = round_dt;
	o->dx = o->dy = o->dz = dx;
	o->mask3 = 0;
	for (int k = 0; k < 9; k++) o->mask9[k] = 0.0;
}

void orc_model_params(double dx, double ifce_width, double xcr0, double xnb0,
                      double meshres, orc_params* o)
{
	orc_model_params_rule(dx, ifce_width, xcr0, xnb0, meshres, 2, 0, o);
}

/* ---- Philox4x32-10, Salmon, Moraes, Dror & Shaw, SC'11 ---- */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
	uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
	uint32_t k0 = key[0], k1 = key[1];
	for (int r = 0; r < 10; r++) {
		if (r > 0) {
			k0 += PHILOX_W0;
			k1 += PHILOX_W1;
		}
		const uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
		const uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
		const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
		const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
		c0 = hi1 ^ c1 ^ k0;
		c1 = lo1;
		c2 = hi0 ^ c3 ^ k1;
		c3 = lo0;
	}
	out[0] = c0;
	out[1] = c1;
	out[2] = c2;
	out[3] = c3;
}

/* 53 random bits -> uniform double in (0, 1]. */
double orc_u53(uint32_t hi, uint32_t lo)
{
	const uint64_t k = ((((uint64_t)hi) << 32) | lo) >> 11;
	return (double)(k + 1) * (1.0 / 9007199254740992.0);
}

/* ---- step semantics with the restated energies ---- */
#define SFN(name) orc_##name
#define E_P(x) orc_p(x)
#define E_PPRIME(x) orc_pprime(x)
#define E_FICT_GAM_CR(a, b, c, d, e) orc_fict(0, 0, a, b, c, d, e)
#define E_FICT_GAM_NB(a, b, c, d, e) orc_fict(0, 1, a, b, c, d, e)
#define E_FICT_DEL_CR(a, b, c, d, e) orc_fict(1, 0, a, b, c, d, e)
#define E_FICT_DEL_NB(a, b, c, d, e) orc_fict(1, 1, a, b, c, d, e)
#define E_FICT_LAV_CR(a, b, c, d, e) orc_fict(2, 0, a, b, c, d, e)
#define E_FICT_LAV_NB(a, b, c, d, e) orc_fict(2, 1, a, b, c, d, e)
#define E_G_GAM(a, b) orc_g(0, a, b)
#define E_G_DEL(a, b) orc_g(1, a, b)
#define E_G_LAV(a, b) orc_g(2, a, b)
#define E_DG_GAM_CR(a, b) orc_dg_gam(0, a, b)
#define E_DG_GAM_NB(a, b) orc_dg_gam(1, a, b)
#define E_D_CRCR(a, b) orc_D(0, 0, a, b)
#define E_D_CRNB(a, b) orc_D(0, 1, a, b)
#define E_D_NBCR(a, b) orc_D(1, 0, a, b)
#define E_D_NBNB(a, b) orc_D(1, 1, a, b)
#define E_DG(ph, c, a, b) orc_dg(ph, c, a, b)
#define E_D2G(ph, i, j) orc_d2g(ph, i, j)
#define E_NUC_PROB orc_nucleation_probability_sphere
#define E_XE_GAM_CR XE[0][0]
#define E_XE_GAM_NB XE[0][1]
#define E_XE_DEL_CR XE[1][0]
#define E_XE_DEL_NB XE[1][1]
#define E_XE_LAV_CR XE[2][0]
#define E_XE_LAV_NB XE[2][1]
#define ORC_RESTRICT restrict
#include "step_impl.h"

/* ---- initial conditions from a recipe ----
 * Per interior cell (x, y, z), interior row-major index c:
 *   u_Cr, u_Nb = orc_u53 of Philox4x32-10 words (0,1), (2,3), counter
 *   (c lo, c hi, 0, 0x49430000), key = seed;
 *   x = matrix + noise (2u - 1);  every band [lo, hi) over x adds enrich - matrix;
 *   particles in order, inside the box |q - floor(c_q)| <= pad on every axis,
 *   pad = ceil(R + 6 (width/2) / dx) + 1: the tanh profile of tanh_interp
 *   (thermo/nucleation.c:12-16) phi = 0.5 - 0.5 tanh(dx (r - R) / (width/2)),
 *   blended as embed_OPC does (src/alloy625.cpp:283-292):
 *   x = p(phi) xe + (1 - p(phi)) x; the particle's phase takes max(phi_old, phi).
 * Plain FP64 with no contraction (this file is built with -ffp-contract=off). */
/* bell_curve of thermo/enrichment.py: A (exp(-x^2/(2 s^2)) - 1) + xe with
 * A set so that the mean over [a, b] is x0 */
static double ic_bell_amplitude(double s, double a, double b, double x0, double xe)
{
	const double I = s * sqrt(M_PI / 2.0) * (erf(b / (s * sqrt(2.0))) - erf(a / (s * sqrt(2.0))));
	return (x0 - xe) / (I / (b - a) - 1.0);
}

static double ic_p(double x)
{
	const double x2 = x * x, x3 = x2 * x;
	return x3 * ((6.0 * x2 - 15.0 * x) + 10.0);
}

void orc_ic_fields(const orc_ic_recipe* r, double* f[4])
{
	const int is3d = r->nz > 1;
	const int nz = is3d ? r->nz : 1;
	const size_t sx = (size_t)r->nx + 2, sy = (size_t)r->ny + 2;
	const double xe[2][2] = {{0.022966218927631978, 0.24984563695705883},
	                         {0.37392129441013022, 0.25826261799015571}};
	const double half_w = 0.5 * r->width;
	const uint32_t key[2] = {(uint32_t)r->seed, (uint32_t)(r->seed >> 32)};
	double bellA[2] = {0.0, 0.0};
	if (r->profile == 1)
		for (int k = 0; k < 2; k++)
			bellA[k] = ic_bell_amplitude(r->bell_sigma[k], r->bell_range[0], r->bell_range[1],
			                             r->matrix[k], r->enrich[k]);
	for (int z = 0; z < nz; z++)
		for (int y = 0; y < r->ny; y++)
			for (int x = 0; x < r->nx; x++) {
				const uint64_t c = ((uint64_t)z * r->ny + y) * (uint64_t)r->nx + x;
				const uint32_t ctr[4] = {(uint32_t)c, (uint32_t)(c >> 32), 0u, 0x49430000u};
				uint32_t w[4];
				orc_philox4x32_10(ctr, key, w);
				double base[2] = {r->matrix[0], r->matrix[1]};
				if (r->profile == 1) {
					/* init_gaussian_enrichment, src/alloy625.cpp:240-255 */
					const double pos = r->dx * ((double)x - r->bell_x0);
					for (int k = 0; k < 2; k++) {
						const double t = pos / r->bell_sigma[k];
						const double v = bellA[k] * (exp(-0.5 * (t * t)) - 1.0) + r->enrich[k];
						base[k] = fmin(1.0, fmax(0.0, v));
					}
				}
				double xcr = base[0] + r->noise * (2.0 * orc_u53(w[0], w[1]) - 1.0);
				double xnb = base[1] + r->noise * (2.0 * orc_u53(w[2], w[3]) - 1.0);
				const double dcr = r->enrich[0] - r->matrix[0], dnb = r->enrich[1] - r->matrix[1];
				for (int b = 0; b < r->n_bands; b++)
					if (x >= r->band[b][0] && x < r->band[b][1]) {
						xcr += dcr;
						xnb += dnb;
					}
				double ph[2] = {0.0, 0.0};
				const int q[3] = {x, y, z};
				for (int k = 0; k < r->n_particles; k++) {
					const double R = r->radius[k];
					/* embed_OPC's box: R + 4 w / dx, truncated (src/alloy625.cpp:275-276) */
					const int pad = r->particle_mode == 1 ? (int)(R + 4.0 * r->width / r->dx)
					                                      : (int)ceil(R + 6.0 * half_w / r->dx) + 1;
					int in = 1;
					double r2 = 0.0;
					for (int d = 0; d < (is3d ? 3 : 2); d++) {
						const int fc = (int)floor(r->centre[k][d]);
						if (q[d] < fc - pad || q[d] > fc + pad) in = 0;
						const double t = (double)q[d] - r->centre[k][d];
						r2 += t * t;
					}
					if (!in) continue;
					const double phi = 0.5 - 0.5 * tanh(r->dx * (sqrt(r2) - R) / half_w);
					const double pp = ic_p(phi), qq = 1.0 - pp;
					const int ph_k = r->phase[k] == 0 ? 0 : 1;
					xcr = pp * xe[ph_k][0] + qq * xcr;
					xnb = pp * xe[ph_k][1] + qq * xnb;
					if (r->particle_mode == 1 || phi > ph[ph_k]) ph[ph_k] = phi;
				}
				const double v[4] = {xcr, xnb, ph[0], ph[1]};
				for (int k = 0; k < 4; k++) {
					double* a = f[k] + (is3d ? (size_t)(z + 1) * sy * sx : 0);
					a[(size_t)(y + 1) * sx + (x + 1)] = v[k];
				}
			}
	/* ghost ring: the mirror of the interior, x then y then z */
	for (int k = 0; k < 4; k++)
		for (int z = 0; z < (is3d ? nz + 2 : 1); z++) {
			double* a = f[k] + (is3d ? (size_t)z * sy * sx : 0);
			for (size_t y = 1; y + 1 < sy; y++) {
				a[y * sx] = a[y * sx + 1];
				a[y * sx + sx - 1] = a[y * sx + sx - 2];
			}
			for (size_t x = 0; x < sx; x++) {
				a[x] = a[sx + x];
				a[(sy - 1) * sx + x] = a[(sy - 2) * sx + x];
			}
		}
	if (is3d)
		for (int k = 0; k < 4; k++) {
			const size_t plane = sy * sx;
			for (size_t i = 0; i < plane; i++) {
				f[k][i] = f[k][plane + i];
				f[k][(size_t)(nz + 1) * plane + i] = f[k][(size_t)nz * plane + i];
			}
		}
}
