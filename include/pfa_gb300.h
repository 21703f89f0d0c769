/*
 * pfa_gb300.h -- extern "C" interface of libpfa_gb300.so.
 *
 * Plain pointers and sizes only.  This is the surface a non-C++ caller
 * (ctypes, cgo, JNI, ...) binds.  Each function below mirrors one
 * reference entry point of usnistgov/phasefield-precipitate-aging with host
 * arrays passed flat instead of through HostData (the C++ drop-in with the
 * reference's own signatures is pfa_reference_abi.h), or adds a capability
 * the reference's loop needs from its caller (multi-step runs, 3D grids,
 * batches of grids).
 *
 * Layout of every 2D field: row-major (ny x nx) doubles with a one-cell ghost
 * ring, nx = Nx + 2, ny = Ny + 2 (src/main.cpp:229-233).  3D fields are
 * (nz x ny x nx) with the same ring.  Field order: x_Cr, x_Nb, phi_delta,
 * phi_laves.
 *
 * Every function returns 0 on success or a PFA_E* code, which also becomes
 * the sticky error word (pfa_last_error).  Nothing here falls back to the
 * CPU: without a usable GPU the calls fail with PFA_ECUDA.
 */
#ifndef PFA_GB300_H
#define PFA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

struct CudaData; /* layout in pfa_reference_abi.h (src/type.h:58-107) */

enum {
	PFA_OK = 0,
	PFA_EINVAL = 1,   /* bad argument or unsupported configuration */
	PFA_ECUDA = 2,    /* a CUDA runtime call failed */
	PFA_ESTATE = 3,   /* CudaData not initialised by this library */
	PFA_EOVERFLOW = 4,/* an event buffer overflowed */
	PFA_ENOMEM = 5    /* device allocation failed */
};

enum { PFA_MODE_FUSED = 0, PFA_MODE_COMPAT = 1 };
/* PFA_FP32: FP32 arithmetic, every field Kahan-compensated with the
 * compensations packed as 16-bit counts (48 bytes per cell update);
 * PFA_FP32_KPHI: the same with FP32 compensations (64 bytes per cell).
 * Both take the 5- or the 9-point mask of src/mesh.cpp:187-213 (any 3x3
 * mask with equal corners, equal left / right and equal upper / lower
 * weights; a step with another mask fails with PFA_EINVAL).  Both index a
 * grid's records (rows of ceil((nx - 2) / 32) * 32, ny - 2 rows; for 3D
 * grids a plane's) with 32-bit integers: from 2^31 records on, switching to
 * them, pfa_batch_add and pfa3d_create fail with PFA_EINVAL. */
enum { PFA_FP64 = 0, PFA_FP32 = 1, PFA_FP32_KPHI = 2 };
enum { PFA_NUC_REFERENCE_GEOMETRY = 0, PFA_NUC_FIXED_GEOMETRY = 1 };
/* Cahn-Hilliard: the reference's constant diffusivity matrix (its loop's
 * form), or its disabled variable-mobility form (see pfa_set_mobility) */
enum { PFA_MOBILITY_CONSTANT = 0, PFA_MOBILITY_VARIABLE = 1 };

/* ---- errors (replaces checkCuda's assert, src/discretization.cu:23-30) ---- */
int pfa_last_error(void);
const char* pfa_error_string(int code);
const char* pfa_last_error_message(void);
void pfa_clear_error(void);

/* ---- device selection (cudaSetDevice for this library's runtime) ---- */
int pfa_set_device(int device);
int pfa_device_count(void);
/* ---- configuration of one CudaData (library-side table) ---- */
int pfa_set_mode(struct CudaData* dev, int mode);
int pfa_set_precision(struct CudaData* dev, int precision);
int pfa_set_nucleation(struct CudaData* dev, uint64_t seed, int geometry);
/* PFA_MOBILITY_VARIABLE: the variable-mobility Cahn-Hilliard the reference
 * wrote and left disabled (mobility_Cr/Nb_kernel src/discretization.cu:175-358,
 * chemical_convolution_Cr/Nb_kernel :618-778, the commented update of
 * composition_kernel :848-856): dx_k/dt = div of 8 coefficient-weighted
 * gradients per component (those of the three phases' fictitious
 * compositions, and of phi_del and phi_lav -- these two along x only, as
 * the reference has them).  Its mobility matrix (d_M_CrCr ..., never
 * defined by the reference) is M = D(x) H_gam^-1 with D(x) the
 * composition-dependent D_CrCr ... D_NbNb and H_gam the gamma curvatures,
 * so that pure gamma diffuses with D(x).  The fused step needs the 5-point
 * mask.  The FP32 forms (pfa_set_precision, 5-point mask with zero weight
 * sum) take it too: with paraboloid energies the phases' fictitious
 * compositions share their diffusion potentials, so the flux is
 * div (D(x) grad x^gamma) with the same face sums, which they evaluate;
 * within 1e-5 of the FP64 form after 1000 steps.  In compat mode (FP64)
 * device_mobilities / mobility_boundaries
 * (and device_laplacian, for a loop that does not call them) compute the
 * coefficients.  No counterpart in the reference's running code. */
int pfa_set_mobility(struct CudaData* dev, int model);

/* ---- mirrors of the reference entry points ---- */
/* init_cuda, src/data.cuh:21-25 / src/data.cu:10-92; mask is nm*nm doubles */
int pfa_init_cuda(struct CudaData* dev, int nx, int ny, int nm, const double* mask,
                  const double* kappa, const double* omega, const double* Lmob,
                  const double* D_Cr, const double* D_Nb, const double* conc_Cr,
                  const double* conc_Nb, const double* phi_del, const double* phi_lav);
/* free_cuda, src/data.cuh:30 / src/data.cu:94-154 */
int pfa_free_cuda(struct CudaData* dev);
/* read_out_result, src/data.cuh:35 / src/data.cu:156-172 */
int pfa_read_out_result(struct CudaData* dev, double* conc_Cr, double* conc_Nb,
                        double* phi_del, double* phi_lav, int nx, int ny);
/* the host-to-device half of init_cuda (src/data.cu:83-91) on a live CudaData */
int pfa_upload_fields(struct CudaData* dev, const double* conc_Cr, const double* conc_Nb,
                      const double* phi_del, const double* phi_lav, int nx, int ny);
/* pfa_read_out_result / pfa_upload_fields without waiting: the copies (and,
 * for the FP32 forms, the layout conversion) are enqueued behind the work
 * already issued on dev and the call returns.  The host buffers must stay
 * valid, and an upload's sources unchanged, until pfa_sync(dev) returns;
 * they overlap other work only when page-locked.  Later work on dev (steps,
 * uploads, read-outs) is ordered after them, so a handle can read out one
 * job, take the next job's fields and step it without waiting in between. */
int pfa_read_out_result_async(struct CudaData* dev, double* conc_Cr, double* conc_Nb,
                              double* phi_del, double* phi_lav, int nx, int ny);
int pfa_upload_fields_async(struct CudaData* dev, const double* conc_Cr, const double* conc_Nb,
                            const double* phi_del, const double* phi_lav, int nx, int ny);
/* src/discretization.cuh:39-111 */
int pfa_device_boundaries(struct CudaData* dev, int nx, int ny, int nm, int bx, int by);
int pfa_device_fictitious(struct CudaData* dev, int nx, int ny, int nm, int bx, int by);
int pfa_fictitious_boundaries(struct CudaData* dev, int nx, int ny, int nm, int bx, int by);
int pfa_device_laplacian(struct CudaData* dev, int nx, int ny, int nm, int bx, int by,
                         double dx, double dy);
int pfa_device_laplacian_boundaries(struct CudaData* dev, int nx, int ny, int nm, int bx, int by);
/* device_mobilities / mobility_boundaries, src/discretization.cuh:46,67
 * (declared, never defined by the reference): compat mode with the variable
 * mobility only, otherwise they return at once */
int pfa_device_mobilities(struct CudaData* dev, int nx, int ny, int nm, int bx, int by);
int pfa_mobility_boundaries(struct CudaData* dev, int nx, int ny, int nm, int bx, int by);
int pfa_device_evolution(struct CudaData* dev, int nx, int ny, int nm, int bx, int by,
                         double alpha, double dt);
int pfa_device_init_prng(struct CudaData* dev, int nx, int ny, int nm, int bx, int by);
int pfa_device_nucleation(struct CudaData* dev, int nx, int ny, int nm, int bx, int by,
                          double sigma_del, double sigma_lav, double unit_a, double ifce_width,
                          double dx, double dy, double dz, double dt);
/* device_dataviz, src/discretization.cuh:116 / src/discretization.cu:1231-1263 */
int pfa_device_dataviz(struct CudaData* dev, double* conc_Cr, double* conc_Nb, double* conc_Ni,
                       double* phi_del, double* phi_lav, double* phi, int nx, int ny);
/* the caller-side pointer swap of src/main.cpp:318-321 */
int pfa_swap(struct CudaData* dev);

/* ---- the update loop of src/main.cpp:285-321 ---- */
/* nsteps x (device_evolution + swap); nucleation after every step whose
 * index k satisfies k % nuc_interval == 0 when nuc_interval > 0
 * (src/main.cpp:307-316), with the nucleation arguments last given to
 * pfa_set_nucleation_args.  Replayed from a captured CUDA graph. */
int pfa_run(struct CudaData* dev, int nsteps, double alpha, double dt);
int pfa_set_nucleation_args(struct CudaData* dev, int nuc_interval, double sigma_del,
                            double sigma_lav, double unit_a, double dx, double dy, double dz,
                            double dt_nuc);
/* pfa_run bracketed by CUDA events on the library's stream; ms = elapsed */
int pfa_run_timed(struct CudaData* dev, int nsteps, double alpha, double dt, float* ms);
/* waits for all work issued on dev, asynchronous read-outs included */
int pfa_sync(struct CudaData* dev);
void* pfa_stream(struct CudaData* dev);
/* number of nucleation events of the last nucleation call, and the events
 * (cell index, phase) in canonical order; returns the count */
int pfa_last_nucleation_events(struct CudaData* dev, int64_t* cells, int32_t* phases, int cap);

/* ---- 3D grids (7-point Laplacian) ----
 * No counterpart in the reference, which is 2D only (src/main.cpp:418-421):
 * the same equations with six-face zero-flux ghost fill.  Fields are
 * (nz x ny x nx) doubles with the ghost ring; params = D_Cr[2], D_Nb[2],
 * kappa[2], omega[2], Lmob[2], alpha, dt (12 doubles, the layout of
 * pfa_model_params' output); dxyz = dx, dy, dz; precision PFA_FP64 or
 * PFA_FP32.  The handle owns its device buffers and stream. */
/* device bytes pfa3d_create allocates: field buffers and nucleation scratch (host-side) */
size_t pfa3d_footprint(int nx, int ny, int nz, int precision);
int pfa3d_create(void** handle, int nx, int ny, int nz, const double* params, const double* dxyz,
                 const double* conc_Cr, const double* conc_Nb, const double* phi_del,
                 const double* phi_lav, int precision);
int pfa3d_run(void* handle, int nsteps);
/* checkpoint / resume of a 3D grid: as pfa_get_counters, pfa_set_counters,
 * pfa_f32_state_bytes, pfa_read_f32_state and pfa_write_f32_state (FP32:
 * A then packed B records, pitch32 x Ny x Nz of each); pfa3d_set_counters
 * after pfa3d_set_nucleation, which resets them */
int pfa3d_get_counters(void* handle, uint64_t* steps, uint64_t* nucleation_calls);
int pfa3d_set_counters(void* handle, uint64_t steps, uint64_t nucleation_calls);
size_t pfa3d_f32_state_bytes(void* handle);
int pfa3d_read_f32_state(void* handle, void* host, size_t bytes);
int pfa3d_write_f32_state(void* handle, const void* host, size_t bytes);
int pfa3d_run_timed(void* handle, int nsteps, float* ms);
int pfa3d_sync(void* handle);  /* wait for the handle's enqueued work */
int pfa3d_read(void* handle, double* conc_Cr, double* conc_Nb, double* phi_del, double* phi_lav);
int pfa3d_upload(void* handle, const double* conc_Cr, const double* conc_Nb,
                 const double* phi_del, const double* phi_lav);
/* pfa3d_read / pfa3d_upload without waiting (as pfa_read_out_result_async /
 * pfa_upload_fields_async): the buffers stay valid, and an upload's sources
 * unchanged, until pfa3d_sync returns; later work on the handle is ordered
 * after them */
int pfa3d_read_async(void* handle, double* conc_Cr, double* conc_Nb, double* phi_del,
                     double* phi_lav);
int pfa3d_upload_async(void* handle, const double* conc_Cr, const double* conc_Nb,
                       const double* phi_del, const double* phi_lav);
int pfa3d_summarize(void* handle, double* out);
/* free energy as pfa_summarize_energy, dV = dx dy dz, gradients in 3D */
int pfa3d_summarize_energy(void* handle, double Omega, double* energy);
/* Philox nucleation on a 3D grid after every step whose index k has
 * k % interval == 0 (interval 0: off), the 2D call's physics with spheres
 * (neighbourhood ball, spherical nucleus and depletion shells); dx, dy, dz
 * and dt_nuc are the nucleation kernel's own (dV = dx dy dz, radii in cells
 * of dx).  Resets the step and call counters.  No counterpart in the
 * reference (2D only). */
int pfa3d_set_nucleation(void* handle, uint64_t seed, int interval, double sigma_del,
                         double sigma_lav, double unit_a, double dx, double dy, double dz,
                         double dt_nuc);
/* events of the last nucleation call, (cell, phase) in ascending cell order,
 * cell = (z ny + y) nx + x in the ghost-ring layout; returns the count */
int pfa3d_last_nucleation_events(void* handle, int64_t* cells, int32_t* phases, int cap);
int pfa3d_destroy(void* handle);
/* For tests of the failure path only: in the next pfa3d_run of this FP32
 * handle, the first CTA of the step kernel neither arms nor issues the
 * staging copy of interior plane `plane`, so its bounded wait runs out
 * (after about a second); the CTA then stops and drains its other copies,
 * and pfa3d_sync / pfa3d_read report PFA_ECUDA ("a TMA staging wait gave
 * up") once and clear it.  That run's result is not meaningful; later runs
 * are normal.  No counterpart in the reference. */
int pfa3d_test_skip_plane(void* handle, int plane);

/* ---- batches of 2D grids (continuous batching) ----
 * No counterpart in the reference, which runs one grid per process
 * (src/main.cpp:285-321).  A batch owns a device arena of arena_bytes and
 * steps every member grid with one launch per time step (FP32 form,
 * packed compensations, 5-point Laplacian); all members share params (the 12
 * doubles of pfa3d_create) and dxy = dx, dy.  Grids join (pfa_batch_add:
 * fields in the reference layout, ny x nx doubles with the ghost ring;
 * PFA_ENOMEM, not printed, when the arena has no room) and leave
 * (pfa_batch_remove) between runs; slot ids are reused.  pfa_batch_add,
 * pfa_batch_remove, pfa_batch_run and pfa_batch_read_async do not wait for
 * the GPU: the fields pass through a staging ring in device memory on copy
 * streams of their own, so one batch's transfers overlap another batch's
 * steps.  pfa_batch_add reads page-locked host arrays asynchronously: keep
 * them unchanged until the next pfa_batch_sync (or pfa_batch_read, which
 * waits); pfa_batch_read_async writes the slot's fields at the state of the
 * runs enqueued before it into page-locked host arrays (null: skipped), valid
 * after the next pfa_batch_sync.  A member advances
 * bit-for-bit as it would alone.  pfa_batch_footprint gives the arena bytes a
 * grid takes.  pfa_batch_tune times the launch shapes (rows per segment,
 * persistent or one warp per unit) on the current members without advancing
 * them and keeps the fastest; pfa_batch_set_launch fixes one. */
size_t pfa_batch_footprint(int nx, int ny);
int pfa_batch_create(void** handle, const double* params, const double* dxy, size_t arena_bytes);
int pfa_batch_add(void* handle, int nx, int ny, const double* conc_Cr, const double* conc_Nb,
                  const double* phi_del, const double* phi_lav, int* slot);
int pfa_batch_remove(void* handle, int slot);
int pfa_batch_read(void* handle, int slot, double* conc_Cr, double* conc_Nb, double* phi_del,
                   double* phi_lav);
int pfa_batch_read_async(void* handle, int slot, double* conc_Cr, double* conc_Nb,
                         double* phi_del, double* phi_lav);
int pfa_batch_run(void* handle, int nsteps);
int pfa_batch_run_timed(void* handle, int nsteps, float* ms);
int pfa_batch_sync(void* handle);
int pfa_batch_summarize(void* handle, int slot, double* out);
int pfa_batch_tune(void* handle, int reps, float* best_ms);
int pfa_batch_set_launch(void* handle, int rows, int persistent, int ctas);
int pfa_batch_get_launch(void* handle, int* rows, int* persistent, int* ctas, int* units);
int pfa_batch_info(void* handle, int* grids, size_t* used_bytes, size_t* arena_bytes);
void* pfa_batch_stream(void* handle);
int pfa_batch_destroy(void* handle);

/* ---- on-device initial conditions ----
 * The reference builds its initial grids on the host (src/alloy625.cpp:170-518:
 * a matrix composition, enriched regions, particles embedded with
 * embed_OPC's tanh profile, :262-294, tanh_interp thermo/nucleation.c:12-16)
 * and writes them to disk for the GPU run.  A recipe describes the same kind
 * of grid so the device builds it in place: no host arrays and no
 * host-to-device copy (the serving layer admits requests this way).
 *   fields = matrix + noise (2u - 1), u uniform in (0, 1] from Philox4x32-10
 *            keyed by seed, counter (cell, 0, 0x49430000), cell = the
 *            interior row-major index, u_Cr from words 0-1, u_Nb from 2-3;
 *   every band adds (enrich - matrix) on interior columns lo <= x < hi
 *            (stripes in 2D, slabs normal to x in 3D; overlapping bands add);
 *   particles in order: inside the box |coord - floor(c)| <= pad on each axis,
 *            pad = ceil(R + 3 width / dx) + 1, phi = 0.5 - 0.5 tanh(dx (r - R)
 *            / (width / 2)), x = p(phi) xe_phase + (1 - p(phi)) x, phi_phase =
 *            max(phi_phase, phi) (r: distance to the centre, in cells);
 *   ghost ring = the zero-flux mirror of the interior.
 * profile 1 replaces matrix_k by init_gaussian_enrichment's bell curve
 * along x (src/alloy625.cpp:210-259, bell_curve of thermo/enrichment.py):
 *   A_k (exp(-(pos / sigma_k)^2 / 2) - 1) + enrich_k, clamped to [0, 1],
 *   pos = dx (x - bell_x0), A_k such that the mean of the unclamped curve
 *   over bell_range [a, b] (m) is matrix_k (noise and bands still apply).
 * particle_mode 1 embeds like embed_OPC (src/alloy625.cpp:262-294): every
 * cell with |q - floor(c_q)| <= int(R + 4 width / dx) on each axis takes the
 * blend and phi_phase = phi (overwritten), in particle order.
 * nz <= 1 makes a 2D grid (centre[k][2] ignored). */
#define PFA_IC_MAX_BANDS 16
#define PFA_IC_MAX_PARTICLES 64
typedef struct pfa_ic_recipe {
	int nx, ny, nz;            /* interior cells */
	double matrix[2];          /* x_Cr, x_Nb */
	double enrich[2];          /* x_Cr, x_Nb inside the bands */
	double noise;              /* half-width of the composition noise */
	uint64_t seed;
	int n_bands;
	int band[PFA_IC_MAX_BANDS][2];             /* interior columns [lo, hi) */
	int n_particles;
	double centre[PFA_IC_MAX_PARTICLES][3];    /* x, y, z in interior cells */
	double radius[PFA_IC_MAX_PARTICLES];       /* cells */
	int phase[PFA_IC_MAX_PARTICLES];           /* 0 delta, 1 laves */
	double dx;                 /* spacing of the tanh profile (m) */
	double width;              /* interface width 2 lambda (m) */
	int profile;               /* 0: matrix + noise + bands; 1: bell curve along x */
	double bell_sigma[2];      /* profile 1: Gaussian widths (m) for x_Cr, x_Nb */
	double bell_range[2];      /* profile 1: [a, b] (m) holding the mean */
	double bell_x0;            /* profile 1: the column (cells) at position 0 */
	int particle_mode;         /* 0: blend, phase = max; 1: embed_OPC's box, phase set */
} pfa_ic_recipe;

/* writes the recipe's four fields into caller-owned device arrays in the
 * reference layout ((ny+2) x (nx+2), or (nz+2) x (ny+2) x (nx+2)), enqueued on
 * `stream` (a cudaStream_t, NULL = default stream) */
int pfa_ic_generate(const pfa_ic_recipe* r, double* conc_Cr, double* conc_Nb, double* phi_del,
                    double* phi_lav, void* stream);
/* pfa_batch_add with the grid built on the device from a 2D recipe */
int pfa_batch_add_ic(void* handle, const pfa_ic_recipe* r, int* slot);
/* pfa3d_create with the grid built on the device from a 3D recipe */
int pfa3d_create_ic(void** handle, const pfa_ic_recipe* r, const double* params,
                    const double* dxyz, int precision);

/* ---- on-device FP64 field summary (src/alloy625.cpp:811-863) ---- */
/* out[5] = mean x_Cr, mean x_Nb, f_gamma, f_delta, f_laves over the interior */
int pfa_summarize(struct CudaData* dev, double* out);

/* The same summary for callers that cannot let a library allocate device
 * memory (a host that owns all device memory through its own pool or a fixed
 * budget, or a step loop that must not see cudaMalloc's implicit device
 * synchronisation).  No counterpart in the reference.  Inputs are four
 * caller-owned device fields in the reference layout (ny rows of nx doubles
 * with the ghost ring); out is a caller-owned device buffer of 5 doubles;
 * the work is enqueued on `stream` (a cudaStream_t, NULL = default stream).
 * Allocates nothing: its scratch is a static device array holding one row of
 * partial sums per grid row, at most 16384 interior rows (ny - 2 <= 16384,
 * else PFA_EINVAL).  The first call on a device looks up that array's device
 * address (cudaGetSymbolAddress), so make it before any stream capture; the
 * address is kept for the life of the process, so do not call it on a device
 * after a cudaDeviceReset of that device.  Calls share the array: calls that
 * overlap on the GPU race.  A CUDA error already pending on the calling
 * thread is reported (PFA_ECUDA) and left pending; nothing is launched. */
int pfa_summarize_fields_noalloc(const double* conc_Cr, const double* conc_Nb,
                                 const double* phi_del, const double* phi_lav, int nx, int ny,
                                 double* out, void* stream);

/* ---- checkpoint / resume ----
 * What a run continues from besides its fields (pfa_read_out_result, and
 * pfa_init_cuda to start again): the step counter (the phase of the
 * nucleation interval) and the nucleation call counter (the Philox counter of
 * the next call); for the FP32 forms also their records, written back
 * exactly, so that a resumed run is bit-identical to an uninterrupted one
 * (FP64 fields alone would re-split every value, which can move a
 * compensation that sits exactly at half an FP32 ulp).  The reference writes
 * its checkpoints as MMSP grid files (src/main.cpp:408), a format this
 * library does not read or write.  pfa_f32_state_bytes is 0 for an FP64
 * handle; pfa_read_f32_state / pfa_write_f32_state take exactly that many
 * bytes and wait for the copies.  pfa_set_counters after
 * pfa_set_nucleation / pfa_set_nucleation_args, which reset them. */
int pfa_get_counters(struct CudaData* dev, uint64_t* steps, uint64_t* nucleation_calls);
int pfa_set_counters(struct CudaData* dev, uint64_t steps, uint64_t nucleation_calls);
size_t pfa_f32_state_bytes(struct CudaData* dev);
int pfa_read_f32_state(struct CudaData* dev, void* host, size_t bytes);
int pfa_write_f32_state(struct CudaData* dev, const void* host, size_t bytes);

/* ---- on-device FP64 free energy (summarize_energy, src/alloy625.cpp:865-919,
 * with gibbs :752-786 and maskedgradient :788-807) ----
 * *energy = sum over interior nodes of dV (g(x, phi) + sum_i kappa_i |grad phi_i|^2),
 * dV = dx dy, Omega the three-phase coefficient (src/parameters.h:37);
 * chem_nrg / grad_nrg (ny x nx, optional, NULL to skip) receive the per-node
 * terms like the reference's host.chem_nrg / grad_nrg (ghost ring 0). */
int pfa_summarize_energy(struct CudaData* dev, double dx, double dy, double Omega, double* energy,
                         double* chem_nrg, double* grad_nrg);

/* ---- model helpers ---- */
/* out[13]: D_Cr[2], D_Nb[2], kappa[2], omega[2], Lmob[2], alpha, dt, rho(D J).
 * dt_rule 0 = the reference's dt (src/main.cpp:260-268, with meshres);
 * dt_rule 1 = half the KKS-aware explicit stability limit. */
int pfa_model_params(double dx, double ifce_width, double xcr0, double xnb0, double meshres,
                     int dim, int dt_rule, double* out);
/* the FP32 fast-path coefficients (44 floats), for tests */
int pfa_model_fast_coef(float* out, int n);
/* Philox4x32-10 on the device for n counters (4 words each) under one
 * 64-bit key, for the generator's known-answer test */
int pfa_philox_block(const uint32_t* ctr, uint64_t key, uint32_t* out, int n);
/* the FP32 form's split of n doubles on the device: hi = nearest FP32,
 * c = float(double(hi) - v) (value = hi - c), for its test */
int pfa_split_block(const double* in, float* hi, float* c, int n);

#ifdef __cplusplus
}
#endif

#endif
