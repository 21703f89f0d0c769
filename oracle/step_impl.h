/*
 * step_impl.h -- the oracle's step, nucleation and summary semantics.
 *
 * TEST INFRASTRUCTURE ONLY (see pfa_oracle.h).
 *
 * This file is included twice: by pfa_oracle.c with the oracle's own
 * restated energies, and by ref_shim.cpp with the reference's compiled
 * thermo/parabola625.c functions.  The includer defines:
 *   SFN(name)            -- symbol prefix for the exported functions
 *   E_P(x), E_PPRIME(x)  -- interpolator p and p'
 *   E_FICT_GAM_CR(...), E_FICT_GAM_NB, E_FICT_DEL_CR, E_FICT_DEL_NB,
 *   E_FICT_LAV_CR, E_FICT_LAV_NB  -- (XCR, XNB, pDel, pGam, pLav)
 *   E_G_GAM, E_G_DEL, E_G_LAV, E_DG_GAM_CR, E_DG_GAM_NB  -- (XCR, XNB)
 *   E_D_CRCR, E_D_CRNB, E_D_NBCR, E_D_NBNB -- composition-dependent diffusivities
 *   E_DG(ph, c, XCR, XNB), E_D2G(ph, i, j) -- dg_<phase>_dx<c> and the constant
 *                          curvatures d2g_<phase>_dx<i><j> (0 gamma, 1 delta,
 *                          2 laves; 0 Cr, 1 Nb)
 *   E_NUC_PROB(...)      -- nucleation_probability_sphere
 *   E_XE_GAM_CR ... E_XE_LAV_NB -- equilibrium compositions (no parentheses)
 * Compiles as C99 and as C++.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef ORC_RESTRICT
#define ORC_RESTRICT
#endif

/* Zero-flux fill of the one-cell halo ring: halo <- adjacent interior.
 * Follows boundary_kernel for nm = 3 (src/discretization.cu:360-394).  The
 * reference fills the four sides concurrently, so its corners are racy; here
 * the side columns are filled first and the rows second, which leaves each
 * corner equal to its diagonal interior neighbour. */
static void SFN(bc2d)(double* f, int nx, int ny)
{
	for (int y = 0; y < ny; y++) {
		f[(size_t)y * nx + 0] = f[(size_t)y * nx + 1];
		f[(size_t)y * nx + nx - 1] = f[(size_t)y * nx + nx - 2];
	}
	for (int x = 0; x < nx; x++) {
		f[x] = f[(size_t)nx + x];
		f[(size_t)(ny - 1) * nx + x] = f[(size_t)(ny - 2) * nx + x];
	}
}

/* 3D analogue (no reference: the reference is 2D only): x faces, then y
 * faces, then z faces, each copying the adjacent interior plane. */
static void SFN(bc3d)(double* f, int nx, int ny, int nz)
{
	const size_t sxy = (size_t)nx * ny;
	for (int z = 0; z < nz; z++)
		for (int y = 0; y < ny; y++) {
			double* row = f + z * sxy + (size_t)y * nx;
			row[0] = row[1];
			row[nx - 1] = row[nx - 2];
		}
	for (int z = 0; z < nz; z++)
		for (int x = 0; x < nx; x++) {
			double* pl = f + z * sxy;
			pl[x] = pl[(size_t)nx + x];
			pl[(size_t)(ny - 1) * nx + x] = pl[(size_t)(ny - 2) * nx + x];
		}
	memcpy(f, f + sxy, sxy * sizeof(double));
	memcpy(f + (size_t)(nz - 1) * sxy, f + (size_t)(nz - 2) * sxy, sxy * sizeof(double));
}

/* Fictitious gamma compositions at every cell, src/discretization.cu:50-74. */
static void SFN(fict_gam_all)(double* const* f, double* ORC_RESTRICT gcr,
                              double* ORC_RESTRICT gnb, size_t n)
{
	const double* cr = f[0];
	const double* nb = f[1];
	const double* pd = f[2];
	const double* pl = f[3];
	long long i;
	#pragma omp parallel for schedule(static)
	for (i = 0; i < (long long)n; i++) {
		const double xCr = cr[i];
		const double xNb = nb[i];
		const double pDel = E_P(pd[i]);
		const double pLav = E_P(pl[i]);
		const double pGam = 1.0 - pDel - pLav;
		gcr[i] = E_FICT_GAM_CR(xCr, xNb, pDel, pGam, pLav);
		gnb[i] = E_FICT_GAM_NB(xCr, xNb, pDel, pGam, pLav);
	}
}

/* Cahn-Hilliard and Allen-Cahn update at one cell, given the four Laplacians.
 * composition_kernel src/discretization.cu:843-865, delta_kernel :888-914,
 * laves_kernel :916-942, allen_cahn_kernel :944-980. */
static void SFN(update_cell)(const orc_params* prm,
                             double xCr, double xNb, double phD, double phL,
                             double lapCr, double lapNb, double lapD, double lapL,
                             double* oCr, double* oNb, double* oD, double* oL)
{
	const double dt = prm->dt;
	*oCr = xCr + dt * (prm->D_Cr[0] * lapCr + prm->D_Cr[1] * lapNb);
	*oNb = xNb + dt * (prm->D_Nb[0] * lapCr + prm->D_Nb[1] * lapNb);

	const double pDel = E_P(phD);
	const double pLav = E_P(phL);
	const double pGam = 1.0 - pDel - pLav;
	const double gam_Cr = E_FICT_GAM_CR(xCr, xNb, pDel, pGam, pLav);
	const double gam_Nb = E_FICT_GAM_NB(xCr, xNb, pDel, pGam, pLav);
	const double gam_nrg = E_G_GAM(gam_Cr, gam_Nb);
	const double dgGdxCr = E_DG_GAM_CR(gam_Cr, gam_Nb);
	const double dgGdxNb = E_DG_GAM_NB(gam_Cr, gam_Nb);

	{
		const double del_Cr = E_FICT_DEL_CR(xCr, xNb, pDel, pGam, pLav);
		const double del_Nb = E_FICT_DEL_NB(xCr, xNb, pDel, pGam, pLav);
		const double del_nrg = E_G_DEL(del_Cr, del_Nb);
		const double gp = gam_nrg - del_nrg - dgGdxCr * (gam_Cr - del_Cr) - dgGdxNb * (gam_Nb - del_Nb);
		const double dF = -E_PPRIME(phD) * gp
		                  + 2.0 * prm->omega[0] * phD * (phD - 1.0) * (2.0 * phD - 1.0)
		                  + 2.0 * prm->alpha * phD * phL * phL
		                  - prm->kappa[0] * lapD;
		*oD = phD - dt * prm->Lmob[0] * dF;
	}
	{
		const double lav_Cr = E_FICT_LAV_CR(xCr, xNb, pDel, pGam, pLav);
		const double lav_Nb = E_FICT_LAV_NB(xCr, xNb, pDel, pGam, pLav);
		const double lav_nrg = E_G_LAV(lav_Cr, lav_Nb);
		const double gp = gam_nrg - lav_nrg - dgGdxCr * (gam_Cr - lav_Cr) - dgGdxNb * (gam_Nb - lav_Nb);
		const double dF = -E_PPRIME(phL) * gp
		                  + 2.0 * prm->omega[1] * phL * (phL - 1.0) * (2.0 * phL - 1.0)
		                  + 2.0 * prm->alpha * phL * phD * phD
		                  - prm->kappa[1] * lapL;
		*oL = phL - dt * prm->Lmob[1] * dF;
	}
}

/* One explicit Euler step, reference sequence src/main.cpp:289-305:
 * boundaries on the old fields, fictitious gamma compositions, their
 * boundaries, 5-point mask convolution (src/discretization.cu:550-603 with the
 * mask of src/mesh.cpp:187-196), Laplacian boundaries, then CH + AC at every
 * cell.  The Laplacians live in new_f until the update overwrites them, as in
 * the reference. */
void SFN(step2d)(double* old_f[4], double* new_f[4], int nx, int ny,
                 const orc_params* prm, double* work)
{
	const size_t n = (size_t)nx * ny;
	double* gcr = work;
	double* gnb = work + n;
	for (int k = 0; k < 4; k++)
		SFN(bc2d)(old_f[k], nx, ny);
	SFN(fict_gam_all)(old_f, gcr, gnb, n);
	SFN(bc2d)(gcr, nx, ny);
	SFN(bc2d)(gnb, nx, ny);

	const double dx = prm->dx, dy = prm->dy;
	const double m_n = 1. / (dy * dy);
	const double m_w = 1. / (dx * dx);
	const double m_c = -2. * (dx * dx + dy * dy) / (dx * dx * dy * dy);
	const double m_e = 1. / (dx * dx);
	const double m_s = 1. / (dy * dy);
	const double* src[4] = {gcr, gnb, old_f[2], old_f[3]};
	const double* m9 = prm->mask9;
	const int general = prm->mask3;
	int y;
	#pragma omp parallel for schedule(static)
	for (y = 1; y < ny - 1; y++) {
		for (int k = 0; k < 4; k++) {
			const double* s = src[k];
			double* d = new_f[k];
			for (int x = 1; x < nx - 1; x++) {
				const size_t i = (size_t)y * nx + x;
				double v = 0.;
				if (general) {
					/* the mask as given, in convolution_kernel's order
					 * (src/discretization.cu:586-595): rows j, columns i */
					for (int j = -1; j <= 1; j++)
						for (int c = -1; c <= 1; c++)
							v += m9[(j + 1) * 3 + (c + 1)] * s[i + (long)j * nx + c];
				} else {
					v += m_n * s[i - nx];
					v += m_w * s[i - 1];
					v += m_c * s[i];
					v += m_e * s[i + 1];
					v += m_s * s[i + nx];
				}
				d[i] = v;
			}
		}
	}
	for (int k = 0; k < 4; k++)
		SFN(bc2d)(new_f[k], nx, ny);

	long long i;
	#pragma omp parallel for schedule(static)
	for (i = 0; i < (long long)n; i++) {
		SFN(update_cell)(prm, old_f[0][i], old_f[1][i], old_f[2][i], old_f[3][i],
		                 new_f[0][i], new_f[1][i], new_f[2][i], new_f[3][i],
		                 &new_f[0][i], &new_f[1][i], &new_f[2][i], &new_f[3][i]);
	}
}

/* ---- variable-mobility Cahn-Hilliard ----
 * The reference's disabled form (mobility_Cr_kernel / mobility_Nb_kernel,
 * src/discretization.cu:175-358, chemical_convolution_Cr/Nb_kernel
 * :618-778, the commented update of composition_kernel :848-856), restated
 * term by term.  The reference never defines the mobility matrix its
 * kernels call (d_M_CrCr ...); here M = D(x) H_gam^-1, with D(x) the
 * composition-dependent diffusivities (thermo/parabola625.c:1860-1894) and
 * H_gam the gamma curvatures, so that in pure gamma the flux is
 * D(x) grad x^gamma.  Per component k the 8 coefficients are, in the
 * reference's order,
 *   gam_k0 = pGam (M_k0 H_gam[0][0] + M_k1 H_gam[.][.]) ... (see below),
 *   phi_del_k = p'(phi_del) (M_k0 (dg_del_Cr - dg_gam_Cr) + M_k1 (dg_del_Nb - dg_gam_Nb)),
 * and the divergence sums, for terms 1-6, the 1D variable-coefficient
 * differences along x and along y, for terms 7-8 along x only (as the
 * reference does).  mob[16]: Cr row gamCrCr gamCrNb delCrCr delCrNb
 * lavCrCr lavCrNb phiDelCr phiLavCr, then the Nb row likewise; fict[6]:
 * x_gam Cr Nb, x_del Cr Nb, x_lav Cr Nb.  All cells of the array. */
static void SFN(mobility_fields)(double* const* f, double* const* fict, double* const* mob,
                                 size_t n)
{
	const double hg00 = E_D2G(0, 0, 0), hg01 = E_D2G(0, 0, 1), hg10 = E_D2G(0, 1, 0),
	             hg11 = E_D2G(0, 1, 1);
	const double det = hg00 * hg11 - hg01 * hg10;
	long long i;
	#pragma omp parallel for schedule(static)
	for (i = 0; i < (long long)n; i++) {
		const double X = f[0][i], Y = f[1][i], phd = f[2][i], phl = f[3][i];
		const double pDel = E_P(phd), pLav = E_P(phl), pGam = 1.0 - pDel - pLav;
		const double xg[2] = {E_FICT_GAM_CR(X, Y, pDel, pGam, pLav), E_FICT_GAM_NB(X, Y, pDel, pGam, pLav)};
		const double xd[2] = {E_FICT_DEL_CR(X, Y, pDel, pGam, pLav), E_FICT_DEL_NB(X, Y, pDel, pGam, pLav)};
		const double xl[2] = {E_FICT_LAV_CR(X, Y, pDel, pGam, pLav), E_FICT_LAV_NB(X, Y, pDel, pGam, pLav)};
		fict[0][i] = xg[0];
		fict[1][i] = xg[1];
		fict[2][i] = xd[0];
		fict[3][i] = xd[1];
		fict[4][i] = xl[0];
		fict[5][i] = xl[1];
		const double D[2][2] = {{E_D_CRCR(X, Y), E_D_CRNB(X, Y)}, {E_D_NBCR(X, Y), E_D_NBNB(X, Y)}};
		double M[2][2];
		for (int k = 0; k < 2; k++) {
			M[k][0] = (D[k][0] * hg11 - D[k][1] * hg10) / det;
			M[k][1] = (D[k][1] * hg00 - D[k][0] * hg01) / det;
		}
		const double pw[3] = {pGam, pDel, pLav};
		const double dgg[2] = {E_DG(0, 0, xg[0], xg[1]), E_DG(0, 1, xg[0], xg[1])};
		const double dgd[2] = {E_DG(1, 0, xd[0], xd[1]), E_DG(1, 1, xd[0], xd[1])};
		const double dgl[2] = {E_DG(2, 0, xl[0], xl[1]), E_DG(2, 1, xl[0], xl[1])};
		const double ppd = E_PPRIME(phd), ppl = E_PPRIME(phl);
		/* Cr row, mobility_Cr_kernel (terms 1-8) */
		for (int ph = 0; ph < 3; ph++) {
			mob[2 * ph][i] = pw[ph] * (M[0][0] * E_D2G(ph, 0, 0) + M[0][1] * E_D2G(ph, 0, 1));
			mob[2 * ph + 1][i] = pw[ph] * (M[0][0] * E_D2G(ph, 1, 0) + M[0][1] * E_D2G(ph, 1, 1));
		}
		mob[6][i] = ppd * (M[0][0] * (dgd[0] - dgg[0]) + M[0][1] * (dgd[1] - dgg[1]));
		mob[7][i] = ppl * (M[0][0] * (dgl[0] - dgg[0]) + M[0][1] * (dgl[1] - dgg[1]));
		/* Nb row, mobility_Nb_kernel (its terms 1-6 read d2g_..._dxNbCr where
		 * the Cr kernel reads ..._dxCrNb: equal, the matrices are symmetric) */
		for (int ph = 0; ph < 3; ph++) {
			mob[8 + 2 * ph][i] = pw[ph] * (M[1][0] * E_D2G(ph, 0, 0) + M[1][1] * E_D2G(ph, 1, 0));
			mob[9 + 2 * ph][i] = pw[ph] * (M[1][0] * E_D2G(ph, 1, 0) + M[1][1] * E_D2G(ph, 1, 1));
		}
		mob[14][i] = ppd * (M[1][0] * (dgd[0] - dgg[0]) + M[1][1] * (dgd[1] - dgg[1]));
		mob[15][i] = ppl * (M[1][0] * (dgl[0] - dgg[0]) + M[1][1] * (dgl[1] - dgg[1]));
	}
}

/* discrete_laplacian, src/discretization.cu:605-616 */
static double SFN(dlap)(double Dl, double Dm, double Dh, double cl, double cm, double ch, double d)
{
	return ((Dh + Dm) * (ch - cm) - (Dm + Dl) * (cm - cl)) / (2.0 * d * d);
}

/* chemical_convolution_<comp>_kernel (src/discretization.cu:618-778) at
 * array cell (x, y): neighbours clamped at the array's edges as there */
static double SFN(chem_div)(double* const* fict, double* const* mobk, const double* phd,
                            const double* phl, int nx, int ny, int x, int y, double dx, double dy)
{
	const size_t mid = (size_t)nx * y + x;
	const size_t lft = x == 0 ? mid : mid - 1;
	const size_t rgt = x == nx - 1 ? mid : mid + 1;
	const size_t bot = y == 0 ? mid : mid - nx;
	const size_t top = y == ny - 1 ? mid : mid + nx;
	/* terms 1-6: (coefficient, composition) pairs */
	const int comp[6] = {0, 1, 2, 3, 4, 5};
	double div = 0.0;
	for (int t = 0; t < 6; t++) {
		const double* D = mobk[t];
		const double* c = fict[comp[t]];
		div += SFN(dlap)(D[lft], D[mid], D[rgt], c[lft], c[mid], c[rgt], dx);
		div += SFN(dlap)(D[bot], D[mid], D[top], c[bot], c[mid], c[top], dy);
	}
	/* terms 7-8: along x only */
	div += SFN(dlap)(mobk[6][lft], mobk[6][mid], mobk[6][rgt], phd[lft], phd[mid], phd[rgt], dx);
	div += SFN(dlap)(mobk[7][lft], mobk[7][mid], mobk[7][rgt], phl[lft], phl[mid], phl[rgt], dx);
	return div;
}

/* One step with the variable-mobility Cahn-Hilliard, in the sequence the
 * reference's loop would run with its mobility calls enabled
 * (src/main.cpp:289-305 with device_mobilities / mobility_boundaries):
 * boundaries, fictitious compositions and their boundaries, mobility
 * coefficients and their boundaries, the divergences of Cr and Nb and the
 * 5-point convolution of the phases into new_f, their boundaries, then the
 * update: x_new = x_old + dt div (the commented form of composition_kernel,
 * src/discretization.cu:848-856) and Allen-Cahn as in the constant form.
 * work: 22 n doubles. */
void SFN(step2d_varmob)(double* old_f[4], double* new_f[4], int nx, int ny,
                        const orc_params* prm, double* work)
{
	const size_t n = (size_t)nx * ny;
	double* fict[6];
	double* mob[16];
	for (int k = 0; k < 6; k++) fict[k] = work + (size_t)k * n;
	for (int k = 0; k < 16; k++) mob[k] = work + (size_t)(6 + k) * n;
	for (int k = 0; k < 4; k++)
		SFN(bc2d)(old_f[k], nx, ny);
	SFN(mobility_fields)(old_f, fict, mob, n);
	for (int k = 0; k < 6; k++)
		SFN(bc2d)(fict[k], nx, ny);
	for (int k = 0; k < 16; k++)
		SFN(bc2d)(mob[k], nx, ny);

	const double dx = prm->dx, dy = prm->dy;
	const double m_n = 1. / (dy * dy);
	const double m_w = 1. / (dx * dx);
	const double m_c = -2. * (dx * dx + dy * dy) / (dx * dx * dy * dy);
	const double m_e = 1. / (dx * dx);
	const double m_s = 1. / (dy * dy);
	int y;
	#pragma omp parallel for schedule(static)
	for (y = 1; y < ny - 1; y++) {
		for (int x = 1; x < nx - 1; x++) {
			const size_t i = (size_t)y * nx + x;
			new_f[0][i] = SFN(chem_div)(fict, mob, old_f[2], old_f[3], nx, ny, x, y, dx, dy);
			new_f[1][i] = SFN(chem_div)(fict, mob + 8, old_f[2], old_f[3], nx, ny, x, y, dx, dy);
			for (int k = 2; k < 4; k++) {
				const double* s = old_f[k];
				double v = 0.;
				v += m_n * s[i - nx];
				v += m_w * s[i - 1];
				v += m_c * s[i];
				v += m_e * s[i + 1];
				v += m_s * s[i + nx];
				new_f[k][i] = v;
			}
		}
	}
	for (int k = 0; k < 4; k++)
		SFN(bc2d)(new_f[k], nx, ny);

	long long i;
	#pragma omp parallel for schedule(static)
	for (i = 0; i < (long long)n; i++) {
		const double divCr = new_f[0][i], divNb = new_f[1][i];
		double oCr, oNb;
		SFN(update_cell)(prm, old_f[0][i], old_f[1][i], old_f[2][i], old_f[3][i],
		                 0.0, 0.0, new_f[2][i], new_f[3][i],
		                 &oCr, &oNb, &new_f[2][i], &new_f[3][i]);
		new_f[0][i] = old_f[0][i] + prm->dt * divCr;
		new_f[1][i] = old_f[1][i] + prm->dt * divNb;
	}
}

void SFN(run2d_varmob)(double* a[4], double* b[4], int nx, int ny, const orc_params* prm,
                       double* work, int nsteps)
{
	for (int s = 0; s < nsteps; s++) {
		SFN(step2d_varmob)(a, b, nx, ny, prm, work);
		for (int k = 0; k < 4; k++) {
			double* t = a[k];
			a[k] = b[k];
			b[k] = t;
		}
	}
}

/* The two divergences of the variable-mobility form (chemical_convolution
 * of Cr and Nb) at the interior cells of a state, after its boundary fill;
 * the ghost ring of out[] is left 0. */
void SFN(chem_div2d)(const double* const f[4], int nx, int ny, double dx, double dy,
                     double* out[2])
{
	const size_t n = (size_t)nx * ny;
	double* fict[6];
	double* mob[16];
	double* g[4];
	double* work = (double*)malloc(26 * n * sizeof(double));
	for (int k = 0; k < 6; k++) fict[k] = work + (size_t)k * n;
	for (int k = 0; k < 16; k++) mob[k] = work + (size_t)(6 + k) * n;
	for (int k = 0; k < 4; k++) {
		g[k] = work + (size_t)(22 + k) * n;
		memcpy(g[k], f[k], n * sizeof(double));
		SFN(bc2d)(g[k], nx, ny);
	}
	SFN(mobility_fields)(g, fict, mob, n);
	for (int k = 0; k < 6; k++) SFN(bc2d)(fict[k], nx, ny);
	for (int k = 0; k < 16; k++) SFN(bc2d)(mob[k], nx, ny);
	memset(out[0], 0, n * sizeof(double));
	memset(out[1], 0, n * sizeof(double));
	for (int y = 1; y < ny - 1; y++)
		for (int x = 1; x < nx - 1; x++) {
			const size_t i = (size_t)y * nx + x;
			out[0][i] = SFN(chem_div)(fict, mob, g[2], g[3], nx, ny, x, y, dx, dy);
			out[1][i] = SFN(chem_div)(fict, mob + 8, g[2], g[3], nx, ny, x, y, dx, dy);
		}
	free(work);
}

/* The fictitious compositions and the 16 mobility coefficients of a state
 * (after its boundary fill), for the golden divergences made with the
 * reference's own chemical_convolution kernels.  f is not modified. */
void SFN(mobility2d)(const double* const f[4], int nx, int ny, double* fict[6], double* mob[16])
{
	const size_t n = (size_t)nx * ny;
	double* g[4];
	for (int k = 0; k < 4; k++) {
		g[k] = (double*)malloc(n * sizeof(double));
		memcpy(g[k], f[k], n * sizeof(double));
		SFN(bc2d)(g[k], nx, ny);
	}
	SFN(mobility_fields)(g, fict, mob, n);
	for (int k = 0; k < 6; k++)
		SFN(bc2d)(fict[k], nx, ny);
	for (int k = 0; k < 16; k++)
		SFN(bc2d)(mob[k], nx, ny);
	for (int k = 0; k < 4; k++)
		free(g[k]);
}

/* nsteps steps with the caller-side pointer swap of src/main.cpp:318-321;
 * on return a[] holds the latest fields (pointers are swapped in place). */
void SFN(run2d)(double* a[4], double* b[4], int nx, int ny, const orc_params* prm,
                double* work, int nsteps)
{
	for (int s = 0; s < nsteps; s++) {
		SFN(step2d)(a, b, nx, ny, prm, work);
		for (int k = 0; k < 4; k++) {
			double* t = a[k];
			a[k] = b[k];
			b[k] = t;
		}
	}
}

/* 3D step: the same sequence with a 7-point Laplacian and six-face zero-flux
 * fill.  The reference has no 3D path (src/main.cpp:418-421); this extends
 * its 2D equations unchanged. */
void SFN(step3d)(double* old_f[4], double* new_f[4], int nx, int ny, int nz,
                 const orc_params* prm, double* work)
{
	const size_t sxy = (size_t)nx * ny;
	const size_t n = sxy * nz;
	double* gcr = work;
	double* gnb = work + n;
	for (int k = 0; k < 4; k++)
		SFN(bc3d)(old_f[k], nx, ny, nz);
	SFN(fict_gam_all)(old_f, gcr, gnb, n);
	SFN(bc3d)(gcr, nx, ny, nz);
	SFN(bc3d)(gnb, nx, ny, nz);

	const double dx = prm->dx, dy = prm->dy, dz = prm->dz;
	const double mx = 1. / (dx * dx), my = 1. / (dy * dy), mz = 1. / (dz * dz);
	const double mc = -2. * (mx + my + mz);
	const double* src[4] = {gcr, gnb, old_f[2], old_f[3]};
	int z;
	#pragma omp parallel for schedule(static)
	for (z = 1; z < nz - 1; z++) {
		for (int k = 0; k < 4; k++) {
			const double* s = src[k];
			double* d = new_f[k];
			for (int y = 1; y < ny - 1; y++)
				for (int x = 1; x < nx - 1; x++) {
					const size_t i = z * sxy + (size_t)y * nx + x;
					double v = 0.;
					v += mz * s[i - sxy];
					v += my * s[i - nx];
					v += mx * s[i - 1];
					v += mc * s[i];
					v += mx * s[i + 1];
					v += my * s[i + nx];
					v += mz * s[i + sxy];
					d[i] = v;
				}
		}
	}
	for (int k = 0; k < 4; k++)
		SFN(bc3d)(new_f[k], nx, ny, nz);

	long long i;
	#pragma omp parallel for schedule(static)
	for (i = 0; i < (long long)n; i++) {
		SFN(update_cell)(prm, old_f[0][i], old_f[1][i], old_f[2][i], old_f[3][i],
		                 new_f[0][i], new_f[1][i], new_f[2][i], new_f[3][i],
		                 &new_f[0][i], &new_f[1][i], &new_f[2][i], &new_f[3][i]);
	}
}

/* Paint one nucleus: embed_OPC_kernel, src/discretization.cu:1046-1077. */
static void SFN(embed)(double* cr, double* nb, double* phi, int nx, int ny,
                       int x, int y, double xCr, double xNb,
                       double par_Cr, double par_Nb, double R_precip)
{
	const double R_dep_Cr = R_precip * sqrt((par_Cr - xCr) / (xCr - E_XE_GAM_CR));
	const double R_dep_Nb = R_precip * sqrt((par_Nb - xNb) / (xNb - E_XE_GAM_NB));
	const long long ntot = (long long)nx * ny;
	for (int i = (int)(-R_precip); i < R_precip; i++) {
		for (int j = (int)(-R_precip); j < R_precip; j++) {
			const long long idn = (long long)nx * (y + j) + (x + i);
			const double r = sqrt((double)(i * i + j * j));
			if (idn >= 0 && idn < ntot) {
				if (r <= R_precip) {
					cr[idn] = par_Cr;
					nb[idn] = par_Nb;
					phi[idn] = 1.;
				} else {
					if (r <= R_dep_Cr)
						cr[idn] = E_XE_GAM_CR;
					if (r <= R_dep_Nb)
						nb[idn] = E_XE_GAM_NB;
				}
			}
		}
	}
}

/* Decide one cell: the per-thread body of nucleation_kernel
 * (src/discretization.cu:1079-1177) evaluated on an unmodified snapshot.
 * Returns a bitmask: bit 0 = delta event, bit 1 = laves event; writes the
 * radii in cells. */
static int SFN(nuc_decide)(double* const* f, int nx, int ny, int x, int y,
                           const orc_nuc_params* np, uint64_t seed, uint64_t call,
                           double* rd, double* rl)
{
	const double dV = np->dx * np->dy * np->dz;
	const double Vatom = 0.25 * np->unit_a * np->unit_a * np->unit_a;
	const double n_gam = dV / Vatom;
	const double R = 1.75e-9 / np->dx;
	const long long ntot = (long long)nx * ny;
	double phi_pre = 0.;
	for (int i = (int)(-R); i < R; i++)
		for (int j = (int)(-R); j < R; j++) {
			const long long idn = (long long)nx * (y + j) + (x + i);
			if (idn >= 0 && idn < ntot && i * i + j * j < R * R)
				phi_pre = fmax(phi_pre, E_P(f[2][idn]) + E_P(f[3][idn]));
		}
	if (!(phi_pre < 1e-10))
		return 0;
	const long long idx = (long long)nx * y + x;
	const double xCr = f[0][idx];
	const double xNb = f[1][idx];
	uint32_t ctr[4] = {(uint32_t)idx, (uint32_t)((uint64_t)idx >> 32),
	                   (uint32_t)call, (uint32_t)(call >> 32)};
	uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
	uint32_t w[4];
	orc_philox4x32_10(ctr, key, w);
	const double u[2] = {orc_u53(w[0], w[1]), orc_u53(w[2], w[3])};
	const double dG = E_G_GAM(xCr, xNb);
	const double dCrCr = E_D_CRCR(xCr, xNb);
	const double dNbNb = E_D_NBNB(xCr, xNb);
	int mask = 0;
	for (int ph = 0; ph < 2; ph++) {
		double Rstar = 0., P = 0.;
		E_NUC_PROB(xCr, xNb, dG, dCrCr, dNbNb, np->sigma[ph], Vatom, n_gam, dV, np->dt, &Rstar, &P);
		if (Rstar > 0.) {
			const double rp = Rstar / np->dx;
			if (P - u[ph] > 0) {
				mask |= 1 << ph;
				if (ph == 0)
					*rd = rp;
				else
					*rl = rp;
			}
		}
	}
	return mask;
}

/* Two-phase nucleation: every interior cell decides on the same snapshot,
 * then events are painted in ascending cell order, delta before laves. */
/* The events of one call in canonical order -- ascending cell, delta before
 * laves -- each with the composition of its cell on the snapshot every
 * decision was taken from (an earlier nucleus painted over a later one's
 * centre does not change the later one's depletion shells); terminated by
 * an entry with phase -1.  Caller frees. */
static orc_nuc_event* SFN(collect_events)(double* const* f, const unsigned char* mask,
                                          const double* rad, size_t n)
{
	size_t m = 0;
	for (size_t i = 0; i < n; i++)
		m += (mask[i] & 1) + ((mask[i] >> 1) & 1);
	orc_nuc_event* ev = (orc_nuc_event*)calloc(m + 1, sizeof(orc_nuc_event));
	size_t k = 0;
	for (size_t i = 0; i < n; i++)
		for (int ph = 0; ph < 2; ph++)
			if (mask[i] & (1 << ph)) {
				ev[k].cell = (int64_t)i;
				ev[k].phase = ph;
				ev[k].xcr = f[0][i];
				ev[k].xnb = f[1][i];
				ev[k].r_precip = rad[2 * i + ph];
				k++;
			}
	ev[m].phase = -1;
	return ev;
}

int SFN(nucleation2d)(double* f[4], int nx, int ny, const orc_nuc_params* np,
                      uint64_t seed, uint64_t call, orc_nuc_event* events, int max_events)
{
	const size_t n = (size_t)nx * ny;
	unsigned char* mask = (unsigned char*)calloc(n, 1);
	double* rad = (double*)calloc(2 * n, sizeof(double));
	int y;
	#pragma omp parallel for schedule(dynamic, 4)
	for (y = 1; y < ny - 1; y++)
		for (int x = 1; x < nx - 1; x++) {
			const size_t i = (size_t)y * nx + x;
			mask[i] = (unsigned char)SFN(nuc_decide)(f, nx, ny, x, y, np, seed, call,
			                                           &rad[2 * i], &rad[2 * i + 1]);
		}
	orc_nuc_event* ev = SFN(collect_events)(f, mask, rad, n);
	int count = 0;
	for (; ev && ev[count].phase >= 0; count++) {
		const orc_nuc_event* e = &ev[count];
		const int x = (int)(e->cell % nx), yy = (int)(e->cell / nx);
		if (e->phase == 0)
			SFN(embed)(f[0], f[1], f[2], nx, ny, x, yy, e->xcr, e->xnb, E_XE_DEL_CR, E_XE_DEL_NB,
			           e->r_precip);
		else
			SFN(embed)(f[0], f[1], f[3], nx, ny, x, yy, e->xcr, e->xnb, E_XE_LAV_CR, E_XE_LAV_NB,
			           e->r_precip);
		if (count < max_events && events)
			events[count] = *e;
	}
	free(ev);
	free(mask);
	free(rad);
	return count;
}

/* Field summary over the interior nodes: mean x_Cr, x_Nb and phase fractions
 * (gamma, delta, laves), src/alloy625.cpp:811-863.  Compensated sums. */
static void SFN(summarize_range)(const double* const* f, size_t nx, size_t ny, size_t nz,
                                 int is3d, double out[5])
{
	double s[5] = {0, 0, 0, 0, 0}, c[5] = {0, 0, 0, 0, 0};
	const size_t z0 = is3d ? 1 : 0, z1 = is3d ? nz - 1 : 1;
	for (size_t z = z0; z < z1; z++)
		for (size_t y = 1; y < ny - 1; y++)
			for (size_t x = 1; x < nx - 1; x++) {
				const size_t i = (z * ny + y) * nx + x;
				double v[5];
				v[0] = f[0][i];
				v[1] = f[1][i];
				v[3] = E_P(f[2][i]);
				v[4] = E_P(f[3][i]);
				v[2] = 1.0;
				v[2] -= v[3];
				v[2] -= v[4];
				for (int k = 0; k < 5; k++) {
					const double yk = v[k] - c[k];
					const double t = s[k] + yk;
					c[k] = (t - s[k]) - yk;
					s[k] = t;
				}
			}
	const double ntot = (double)(nx - 2) * (double)(ny - 2) * (is3d ? (double)(nz - 2) : 1.0);
	for (int k = 0; k < 5; k++)
		out[k] = s[k] / ntot;
}

void SFN(summarize2d)(const double* f[4], int nx, int ny, double out[5])
{
	SFN(summarize_range)(f, nx, ny, 1, 0, out);
}

void SFN(summarize3d)(const double* f[4], int nx, int ny, int nz, double out[5])
{
	SFN(summarize_range)(f, nx, ny, nz, 1, out);
}

/* Free energy of the grid, src/alloy625.cpp:752-786 (gibbs), :788-807
 * (maskedgradient) and :865-919 (summarize_energy), 2D: per interior node
 *   chem = dV * ( pGam g_gam(x^gam) + pDel g_del(x^del) + pLav g_lav(x^lav)
 *                 + sum_i omega_i phi_i^2 (1 - phi_i)^2
 *                 + 2 Omega phi_del^2 phi_lav^2 )
 *   grad = dV * sum_i kappa_i |grad phi_i|^2, central differences
 *          (phi(x+1) - phi(x-1)) / (2 dx) reading the ghost ring at the edges,
 * dV = dx dy.  chem / grad (nx*ny, optional) receive the per-node values at
 * the node's index (ghost ring untouched); returns the sum over the nodes of
 * chem + grad, accumulated in row-major order. */
double SFN(energy2d)(const double* f[4], int nx, int ny, double dx, double dy,
                     const double kappa[2], const double omega[2], double Omega,
                     double* chem, double* grad)
{
	const double dV = dx * dy;
	const double wx = 1.0 / (2.0 * dx), wy = 1.0 / (2.0 * dy);
	double energy = 0.0;
	for (int y = 1; y < ny - 1; y++)
		for (int x = 1; x < nx - 1; x++) {
			const size_t i = (size_t)y * nx + x;
			const double xCr = f[0][i], xNb = f[1][i];
			const double phi[2] = {f[2][i], f[3][i]};
			const double pDel = E_P(phi[0]);
			const double pLav = E_P(phi[1]);
			const double pGam = 1.0 - pDel - pLav;
			const double gCr = E_FICT_GAM_CR(xCr, xNb, pDel, pGam, pLav);
			const double gNb = E_FICT_GAM_NB(xCr, xNb, pDel, pGam, pLav);
			const double dCr = E_FICT_DEL_CR(xCr, xNb, pDel, pGam, pLav);
			const double dNb = E_FICT_DEL_NB(xCr, xNb, pDel, pGam, pLav);
			const double lCr = E_FICT_LAV_CR(xCr, xNb, pDel, pGam, pLav);
			const double lNb = E_FICT_LAV_NB(xCr, xNb, pDel, pGam, pLav);
			const double sq[2] = {phi[0] * phi[0], phi[1] * phi[1]};
			double g = pGam * E_G_GAM(gCr, gNb);
			g += pDel * E_G_DEL(dCr, dNb);
			g += pLav * E_G_LAV(lCr, lNb);
			for (int k = 0; k < 2; k++) {
				const double u = 1.0 - phi[k];
				g += omega[k] * sq[k] * (u * u);
			}
			g += 2.0 * Omega * sq[0] * sq[1];
			double ge = 0.0;
			for (int k = 0; k < 2; k++) {
				const double* p = f[2 + k];
				const double gx = wx * (p[i + 1] - p[i - 1]);
				const double gy = wy * (p[i + nx] - p[i - nx]);
				ge += kappa[k] * (gx * gx + gy * gy);
			}
			const double c = g * dV, e = ge * dV;
			if (chem) chem[i] = c;
			if (grad) grad[i] = e;
			energy += c + e;
		}
	return energy;
}

/* ---- 3D nucleation (no counterpart in the reference, which is 2D only) ----
 * The 2D semantics above with spheres: the neighbourhood scan covers
 * i^2 + j^2 + k^2 < R^2 and the nucleus and its depletion shells are
 * spheres; offsets that leave the array along any axis are skipped (the 2D
 * reference's row wrap-around is a property of its linear indexing that a
 * 3D extension does not inherit).  Cell index: (z ny + y) nx + x in the
 * ghost-ring layout. */
static void SFN(embed3d)(double* cr, double* nb, double* phi, int nx, int ny, int nz,
                         int x, int y, int z, double xCr, double xNb,
                         double par_Cr, double par_Nb, double R_precip)
{
	const double R_dep_Cr = R_precip * sqrt((par_Cr - xCr) / (xCr - E_XE_GAM_CR));
	const double R_dep_Nb = R_precip * sqrt((par_Nb - xNb) / (xNb - E_XE_GAM_NB));
	for (int k = (int)(-R_precip); k < R_precip; k++)
		for (int j = (int)(-R_precip); j < R_precip; j++)
			for (int i = (int)(-R_precip); i < R_precip; i++) {
				const int xx = x + i, yy = y + j, zz = z + k;
				if (xx < 0 || xx >= nx || yy < 0 || yy >= ny || zz < 0 || zz >= nz)
					continue;
				const size_t idn = ((size_t)zz * ny + yy) * nx + xx;
				const double r = sqrt((double)(i * i + j * j + k * k));
				if (r <= R_precip) {
					cr[idn] = par_Cr;
					nb[idn] = par_Nb;
					phi[idn] = 1.;
				} else {
					if (r <= R_dep_Cr)
						cr[idn] = E_XE_GAM_CR;
					if (r <= R_dep_Nb)
						nb[idn] = E_XE_GAM_NB;
				}
			}
}

static int SFN(nuc_decide3d)(double* const* f, int nx, int ny, int nz, int x, int y, int z,
                             const orc_nuc_params* np, uint64_t seed, uint64_t call,
                             double* rd, double* rl)
{
	const double dV = np->dx * np->dy * np->dz;
	const double Vatom = 0.25 * np->unit_a * np->unit_a * np->unit_a;
	const double n_gam = dV / Vatom;
	const double R = 1.75e-9 / np->dx;
	double phi_pre = 0.;
	for (int k = (int)(-R); k < R; k++)
		for (int j = (int)(-R); j < R; j++)
			for (int i = (int)(-R); i < R; i++) {
				const int xx = x + i, yy = y + j, zz = z + k;
				if (xx < 0 || xx >= nx || yy < 0 || yy >= ny || zz < 0 || zz >= nz)
					continue;
				if (i * i + j * j + k * k < R * R) {
					const size_t idn = ((size_t)zz * ny + yy) * nx + xx;
					phi_pre = fmax(phi_pre, E_P(f[2][idn]) + E_P(f[3][idn]));
				}
			}
	if (!(phi_pre < 1e-10))
		return 0;
	const long long idx = ((long long)z * ny + y) * nx + x;
	const double xCr = f[0][idx];
	const double xNb = f[1][idx];
	uint32_t ctr[4] = {(uint32_t)idx, (uint32_t)((uint64_t)idx >> 32),
	                   (uint32_t)call, (uint32_t)(call >> 32)};
	uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
	uint32_t w[4];
	orc_philox4x32_10(ctr, key, w);
	const double u[2] = {orc_u53(w[0], w[1]), orc_u53(w[2], w[3])};
	const double dG = E_G_GAM(xCr, xNb);
	const double dCrCr = E_D_CRCR(xCr, xNb);
	const double dNbNb = E_D_NBNB(xCr, xNb);
	int mask = 0;
	for (int ph = 0; ph < 2; ph++) {
		double Rstar = 0., P = 0.;
		E_NUC_PROB(xCr, xNb, dG, dCrCr, dNbNb, np->sigma[ph], Vatom, n_gam, dV, np->dt, &Rstar, &P);
		if (Rstar > 0.) {
			const double rp = Rstar / np->dx;
			if (P - u[ph] > 0) {
				mask |= 1 << ph;
				if (ph == 0)
					*rd = rp;
				else
					*rl = rp;
			}
		}
	}
	return mask;
}

int SFN(nucleation3d)(double* f[4], int nx, int ny, int nz, const orc_nuc_params* np,
                      uint64_t seed, uint64_t call, orc_nuc_event* events, int max_events)
{
	const size_t n = (size_t)nx * ny * nz;
	unsigned char* mask = (unsigned char*)calloc(n, 1);
	double* rad = (double*)calloc(2 * n, sizeof(double));
	int z;
	#pragma omp parallel for schedule(dynamic, 1)
	for (z = 1; z < nz - 1; z++)
		for (int y = 1; y < ny - 1; y++)
			for (int x = 1; x < nx - 1; x++) {
				const size_t i = ((size_t)z * ny + y) * nx + x;
				mask[i] = (unsigned char)SFN(nuc_decide3d)(f, nx, ny, nz, x, y, z, np, seed, call,
				                                             &rad[2 * i], &rad[2 * i + 1]);
			}
	orc_nuc_event* ev = SFN(collect_events)(f, mask, rad, n);
	int count = 0;
	for (; ev && ev[count].phase >= 0; count++) {
		const orc_nuc_event* e = &ev[count];
		const int x = (int)(e->cell % nx), y = (int)((e->cell / nx) % ny);
		const int zz = (int)(e->cell / ((int64_t)nx * ny));
		if (e->phase == 0)
			SFN(embed3d)(f[0], f[1], f[2], nx, ny, nz, x, y, zz, e->xcr, e->xnb, E_XE_DEL_CR,
			             E_XE_DEL_NB, e->r_precip);
		else
			SFN(embed3d)(f[0], f[1], f[3], nx, ny, nz, x, y, zz, e->xcr, e->xnb, E_XE_LAV_CR,
			             E_XE_LAV_NB, e->r_precip);
		if (count < max_events && events)
			events[count] = *e;
	}
	free(ev);
	free(mask);
	free(rad);
	return count;
}
