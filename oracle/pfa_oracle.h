/*
 * pfa_oracle.h -- CPU oracle for the KKS Cr-Nb-Ni explicit time step.
 *
 * TEST INFRASTRUCTURE ONLY.  The tests, the smoke check and the
 * CPU-baseline leg of the benchmark load it to check the CUDA library's
 * results against it (or to time it beside the library).  The product never links,
 * loads or calls it.
 *
 * It restates, in plain FP64 C, the semantics of the reference's step
 * (usnistgov/phasefield-precipitate-aging, src/discretization.cu:50-1020),
 * nucleation (src/discretization.cu:1046-1209, thermo/nucleation.c:30-69),
 * field summary (src/alloy625.cpp:811-863) and the generated paraboloid
 * energies (thermo/parabola625.c).  Every function cites the lines it follows.
 *
 * Layout: every 2D field is a row-major (ny x nx) array with a one-cell halo
 * ring, nx = Nx + 2, ny = Ny + 2, index = nx*y + x (src/main.cpp:229-233,
 * src/discretization.cu:63).  3D fields are (nz x ny x nx) with the same ring.
 * Field order everywhere: 0 = x_Cr, 1 = x_Nb, 2 = phi_delta, 3 = phi_laves.
 */
#ifndef PFA_ORACLE_H
#define PFA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
	double D_Cr[2];   /* row of the constant diffusion matrix for Cr: [D_CrCr, D_CrNb] */
	double D_Nb[2];   /* [D_NbCr, D_NbNb] */
	double kappa[2];  /* gradient energy coefficients (delta, laves), J/m */
	double omega[2];  /* double-well heights, J/m^3 */
	double Lmob[2];   /* Allen-Cahn mobilities */
	double alpha;     /* three-phase penalty (Omega), J/m^3 */
	double dt;        /* time step, s */
	double dx, dy, dz;/* grid spacing, m (dz unused in 2D) */
	int mask3;        /* 2D step: 0 = the 5-point mask of dx, dy (src/mesh.cpp:187-196);
	                     1 = convolve mask9 as given, like the reference's
	                     convolution_kernel (src/discretization.cu:550-603) */
	double mask9[9];  /* 3 x 3 mask, rows y-1 .. y+1, columns x-1 .. x+1 */
} orc_params;

typedef struct {
	double sigma[2];  /* interfacial energies (delta, laves), J/m^2 */
	double unit_a;    /* lattice constant used for the atomic volume, m */
	double dx, dy, dz;/* spacing seen by the nucleation kernel (the reference
	                     wrapper passes dx*nx, dy*ny here: the caller decides) */
	double dt;        /* nucleation interval in seconds */
} orc_nuc_params;

typedef struct {
	int64_t cell;     /* linear index nx*y + x in the halo layout */
	int32_t phase;    /* 0 = delta, 1 = laves */
	int32_t pad;
	double xcr, xnb;  /* composition at the nucleus centre before painting */
	double r_precip;  /* nucleus radius in cells */
} orc_nuc_event;

/* ---- model constants (thermo/parabola625.c:38-117,299-315) ---- */
double orc_kT(void);
double orc_RT(void);
double orc_Vm(void);
double orc_xe(int phase, int comp); /* phase 0=gam 1=del 2=lav, comp 0=Cr 1=Nb */

/* ---- pointwise energies ---- */
double orc_p(double x);
double orc_pprime(double x);
double orc_fict(int phase, int comp, double xcr, double xnb,
                double pdel, double pgam, double plav);
double orc_g(int phase, double xcr, double xnb);
double orc_dg_gam(int comp, double xcr, double xnb);
double orc_D(int row, int col, double xcr, double xnb);
double orc_dg(int phase, int comp, double xcr, double xnb);
double orc_d2g(int phase, int i, int j);
void orc_nucleation_probability_sphere(double xcr, double xnb, double dG_chem,
                                       double D_CrCr, double D_NbNb, double sigma,
                                       double Vatom, double n_gam, double dV, double dt,
                                       double* Rstar, double* P_nuc);
void orc_model_params(double dx, double ifce_width, double xcr0, double xnb0,
                      double meshres, orc_params* out);
void orc_model_params_rule(double dx, double ifce_width, double xcr0, double xnb0,
                           double meshres, int dim, int dt_rule, orc_params* out);
double orc_kks_diffusivity(const double Dcr[2], const double Dnb[2]);

/* ---- Philox4x32-10 (Salmon et al., SC'11) ---- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double orc_u53(uint32_t hi, uint32_t lo);

/* ---- steps (modify the halo of `old` like the reference's boundary fill) ---- */
void orc_step2d(double* old_f[4], double* new_f[4], int nx, int ny,
                const orc_params* prm, double* work /* 2*nx*ny doubles */);
void orc_run2d(double* a[4], double* b[4], int nx, int ny, const orc_params* prm,
               double* work, int nsteps);
/* variable-mobility Cahn-Hilliard (the reference's disabled mobility kernels),
 * work = 22*nx*ny doubles; orc_mobility2d: the 6 fictitious compositions and
 * the 16 mobility coefficients of a state (after its boundary fill) */
void orc_step2d_varmob(double* old_f[4], double* new_f[4], int nx, int ny,
                       const orc_params* prm, double* work);
void orc_run2d_varmob(double* a[4], double* b[4], int nx, int ny, const orc_params* prm,
                      double* work, int nsteps);
void orc_mobility2d(const double* const f[4], int nx, int ny, double* fict[6], double* mob[16]);
void orc_chem_div2d(const double* const f[4], int nx, int ny, double dx, double dy,
                    double* out[2]);
void orc_step3d(double* old_f[4], double* new_f[4], int nx, int ny, int nz,
                const orc_params* prm, double* work /* 2*nx*ny*nz doubles */);

/* ---- nucleation: deterministic two-phase form of the reference kernel ---- */
int orc_nucleation2d(double* f[4], int nx, int ny, const orc_nuc_params* np,
                     uint64_t seed, uint64_t call_index,
                     orc_nuc_event* events, int max_events);
/* 3D form (spheres; cell = (z ny + y) nx + x in the ghost-ring layout) */
int orc_nucleation3d(double* f[4], int nx, int ny, int nz, const orc_nuc_params* np,
                     uint64_t seed, uint64_t call_index,
                     orc_nuc_event* events, int max_events);

/* ---- reductions (src/alloy625.cpp:811-863) ---- */
void orc_summarize2d(const double* f[4], int nx, int ny, double out[5]);
void orc_summarize3d(const double* f[4], int nx, int ny, int nz, double out[5]);

/* ---- free energy (src/alloy625.cpp:752-807,865-919) ---- */
double orc_energy2d(const double* f[4], int nx, int ny, double dx, double dy,
                    const double kappa[2], const double omega[2], double Omega,
                    double* chem, double* grad);

/* ---- initial conditions from a recipe (the grids the reference builds on
 * the host, src/alloy625.cpp:170-518, embed_OPC :262-294; the layout matches
 * the library's recipe struct field for field) ---- */
#define ORC_IC_MAX_BANDS 16
#define ORC_IC_MAX_PARTICLES 64
typedef struct {
	int nx, ny, nz;
	double matrix[2], enrich[2], noise;
	uint64_t seed;
	int n_bands;
	int band[ORC_IC_MAX_BANDS][2];
	int n_particles;
	double centre[ORC_IC_MAX_PARTICLES][3];
	double radius[ORC_IC_MAX_PARTICLES];
	int phase[ORC_IC_MAX_PARTICLES];
	double dx, width;
	int profile;               /* 1: init_gaussian_enrichment's bell curve along x */
	double bell_sigma[2], bell_range[2], bell_x0;
	int particle_mode;         /* 1: embed_OPC's square box, phase overwritten */
} orc_ic_recipe;
/* fields in the ghost-ring layout ((ny+2) x (nx+2), or (nz+2) x (ny+2) x (nx+2)
 * when nz > 1), ghost ring = the mirror of the interior */
void orc_ic_fields(const orc_ic_recipe* r, double* f[4]);

#ifdef __cplusplus
}
#endif

#endif
