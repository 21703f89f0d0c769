/*
 * ref_shim.cpp -- links the oracle's step semantics to the reference's own
 * compiled energy functions (thermo/parabola625.c, thermo/nucleation.c of
 * usnistgov/phasefield-precipitate-aging, compiled from where they lie by
 * oracle/Makefile into oracle/_ref/).
 *
 * TEST INFRASTRUCTURE ONLY.  Used in the build container to make the golden
 * vectors under tests/golden (tests/golden/make_golden.py); it pins the
 * oracle's restated energy tables against the reference's code.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "parabola625.h"
#include "nucleation.h"
#include "pfa_oracle.h"

extern "C" {

double ref_p(double x) { return p(x); }
double ref_pprime(double x) { return pPrime(x); }
double ref_tanh_interp(double r, double w) { return tanh_interp(r, w); }

/* the reference's dg_<phase>_dx<comp> and d2g_<phase>_dx<i><j> by index
 * (phase 0 gamma, 1 delta, 2 laves; comp 0 Cr, 1 Nb) */
double ref_dg_phase(int phase, int comp, double a, double b)
{
	switch (phase * 2 + comp) {
	case 0: return dg_gam_dxCr(a, b);
	case 1: return dg_gam_dxNb(a, b);
	case 2: return dg_del_dxCr(a, b);
	case 3: return dg_del_dxNb(a, b);
	case 4: return dg_lav_dxCr(a, b);
	default: return dg_lav_dxNb(a, b);
	}
}

double ref_d2g_phase(int phase, int i, int j)
{
	switch (phase * 4 + i * 2 + j) {
	case 0: return d2g_gam_dxCrCr();
	case 1: return d2g_gam_dxCrNb();
	case 2: return d2g_gam_dxNbCr();
	case 3: return d2g_gam_dxNbNb();
	case 4: return d2g_del_dxCrCr();
	case 5: return d2g_del_dxCrNb();
	case 6: return d2g_del_dxNbCr();
	case 7: return d2g_del_dxNbNb();
	case 8: return d2g_lav_dxCrCr();
	case 9: return d2g_lav_dxCrNb();
	case 10: return d2g_lav_dxNbCr();
	default: return d2g_lav_dxNbNb();
	}
}

/* embed_OPC (src/alloy625.cpp:262-294) on a 2D grid in the ghost-ring layout
 * (rows of nx doubles, f = x_Cr, x_Nb, phi_del, phi_lav), seed centre
 * (cx, cy) in array coordinates, restated without MMSP: over the box
 * |i|, |j| <= int(R + 4 w / meshres), phi = tanh_interp(meshres (r - R), w / 2)
 * with the reference's compiled tanh_interp and p, phase field pid (2 or 3)
 * set to phi, compositions blended toward (par_cr, par_nb) by p(phi). */
void ref_embed_opc(double* f[4], int nx, int ny, int cx, int cy, double par_cr, double par_nb,
                   double R_precip, int pid, double meshres, double ifce_width)
{
	const int R = (int)(R_precip + 4 * ifce_width / meshres);
	for (int i = -R; i < R + 1; i++)
		for (int j = -R; j < R + 1; j++) {
			const int x = cx + i, y = cy + j;
			if (x < 0 || x >= nx || y < 0 || y >= ny) continue;
			const size_t k = (size_t)y * nx + x;
			const double xCr = f[0][k], xNb = f[1][k];
			const double r = sqrt((double)(i * i + j * j));
			const double z = meshres * (r - R_precip);
			const double phi = tanh_interp(z, ifce_width / 2);
			const double pgam = 1.0 - p(phi);
			f[pid][k] = phi;
			f[0][k] = p(phi) * par_cr + pgam * xCr;
			f[1][k] = p(phi) * par_nb + pgam * xNb;
		}
}

double ref_fict(int phase, int comp, double a, double b, double c, double d, double e)
{
	switch (phase * 2 + comp) {
	case 0: return fict_gam_Cr(a, b, c, d, e);
	case 1: return fict_gam_Nb(a, b, c, d, e);
	case 2: return fict_del_Cr(a, b, c, d, e);
	case 3: return fict_del_Nb(a, b, c, d, e);
	case 4: return fict_lav_Cr(a, b, c, d, e);
	default: return fict_lav_Nb(a, b, c, d, e);
	}
}

double ref_g(int phase, double a, double b)
{
	return phase == 0 ? g_gam(a, b) : (phase == 1 ? g_del(a, b) : g_lav(a, b));
}

double ref_dg(int phase, int comp, double a, double b)
{
	switch (phase * 2 + comp) {
	case 0: return dg_gam_dxCr(a, b);
	case 1: return dg_gam_dxNb(a, b);
	case 2: return dg_del_dxCr(a, b);
	case 3: return dg_del_dxNb(a, b);
	case 4: return dg_lav_dxCr(a, b);
	default: return dg_lav_dxNb(a, b);
	}
}

double ref_D(int row, int col, double a, double b)
{
	switch (row * 2 + col) {
	case 0: return D_CrCr(a, b);
	case 1: return D_CrNb(a, b);
	case 2: return D_NbCr(a, b);
	default: return D_NbNb(a, b);
	}
}

double ref_xe(int phase, int comp)
{
	switch (phase * 2 + comp) {
	case 0: return xe_gam_Cr();
	case 1: return xe_gam_Nb();
	case 2: return xe_del_Cr();
	case 3: return xe_del_Nb();
	case 4: return xe_lav_Cr();
	default: return xe_lav_Nb();
	}
}

double ref_kT(void) { return kT(); }
double ref_RT(void) { return RT(); }
double ref_Vm(void) { return Vm(); }

void ref_nucleation_probability_sphere(double xCr, double xNb, double dG, double dcc, double dnn,
                                       double sigma, double Vatom, double n_gam, double dV,
                                       double dt, double* Rstar, double* P)
{
	nucleation_probability_sphere(xCr, xNb, dG, dcc, dnn, sigma, Vatom, n_gam, dV, dt, Rstar, P);
}

/* Philox is the project's own (no counterpart in the reference). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double orc_u53(uint32_t hi, uint32_t lo);

} /* extern "C" */

static void nuc_prob_ref(double xCr, double xNb, double dG, double dcc, double dnn, double sigma,
                         double Vatom, double n_gam, double dV, double dt, double* R, double* P)
{
	nucleation_probability_sphere(xCr, xNb, dG, dcc, dnn, sigma, Vatom, n_gam, dV, dt, R, P);
}

extern "C" {
#define SFN(name) ref_##name
#define E_P(x) p(x)
#define E_PPRIME(x) pPrime(x)
#define E_FICT_GAM_CR fict_gam_Cr
#define E_FICT_GAM_NB fict_gam_Nb
#define E_FICT_DEL_CR fict_del_Cr
#define E_FICT_DEL_NB fict_del_Nb
#define E_FICT_LAV_CR fict_lav_Cr
#define E_FICT_LAV_NB fict_lav_Nb
#define E_G_GAM g_gam
#define E_G_DEL g_del
#define E_G_LAV g_lav
#define E_DG_GAM_CR dg_gam_dxCr
#define E_DG_GAM_NB dg_gam_dxNb
#define E_D_CRCR D_CrCr
#define E_D_CRNB D_CrNb
#define E_D_NBCR D_NbCr
#define E_D_NBNB D_NbNb
#define E_DG(ph, c, a, b) ref_dg_phase(ph, c, a, b)
#define E_D2G(ph, i, j) ref_d2g_phase(ph, i, j)
#define E_NUC_PROB nuc_prob_ref
#define E_XE_GAM_CR xe_gam_Cr()
#define E_XE_GAM_NB xe_gam_Nb()
#define E_XE_DEL_CR xe_del_Cr()
#define E_XE_DEL_NB xe_del_Nb()
#define E_XE_LAV_CR xe_lav_Cr()
#define E_XE_LAV_NB xe_lav_Nb()
#define ORC_RESTRICT __restrict__
#include "step_impl.h"
}
