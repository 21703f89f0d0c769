/*
 * pfa_reference_abi.h -- the reference's own GPU entry points, as exported by
 * libpfa_gb300.so.
 *
 * libpfa_gb300 is a drop-in for the CUDA objects of
 * usnistgov/phasefield-precipitate-aging (src/data.cu, src/discretization.cu,
 * src/nucleation.cu, src/parabola625.cu): the caller (src/main.cpp) keeps
 * its own headers and links this library instead.  The declarations below
 * repeat the reference's host interface with identical C++ signatures and
 * structure layouts, so the mangled symbols and the caller-allocated
 * CudaData / HostData match.
 *
 * Semantics that differ from the reference are listed per function.  All
 * functions are synchronous from the caller's view, as in the reference.
 * Failures print "CUDA Runtime Error: <message>" to stderr (checkCuda
 * behaviour, src/discretization.cu:23-30) and set the sticky error word read
 * by pfa_last_error() (pfa_gb300.h).
 */
#ifndef PFA_REFERENCE_ABI_H
#define PFA_REFERENCE_ABI_H

#include <cuda_runtime.h>

/* src/type.h:13-23 */
#ifndef NP
#define NP 2
#endif
#ifndef NC
#define NC 2
#endif
typedef double fp_t;

/* src/mesh.h:49-54 */
#ifndef MAX_MASK_W
#define MAX_MASK_W 5
#endif
#ifndef MAX_MASK_H
#define MAX_MASK_H 5
#endif

/* Same type as curand's curandState (an XORWOW state); the library never
 * dereferences it and leaves CudaData::prng NULL (nucleation draws come from
 * a counter-based Philox generator that needs no per-cell state). */
struct curandStateXORWOW;
typedef struct curandStateXORWOW curandState;

/* src/type.h:28-53 (host arrays; row pointers over one contiguous block) */
struct HostData {
	fp_t** mask_lap;
	fp_t** conc_Ni;
	fp_t** phi;

	fp_t** chem_nrg;
	fp_t** grad_nrg;

	fp_t** conc_Cr_old;
	fp_t** conc_Cr_new;
	fp_t** conc_Cr_lap;
	fp_t** conc_Cr_gam;

	fp_t** conc_Nb_old;
	fp_t** conc_Nb_new;
	fp_t** conc_Nb_lap;
	fp_t** conc_Nb_gam;

	fp_t** phi_del_old;
	fp_t** phi_del_new;
	fp_t** phi_del_lap;

	fp_t** phi_lav_old;
	fp_t** phi_lav_new;
	fp_t** phi_lav_lap;
};

/* src/type.h:58-107 (device state; the caller swaps *_old / *_new) */
struct CudaData {
	curandState* prng;
	cudaStream_t str_A, str_B, str_C, str_D;
	cudaEvent_t ev_A, ev_B, ev_C, ev_D;

	fp_t* conc_Ni;
	fp_t* phi;

	fp_t* conc_Cr_old;
	fp_t* conc_Cr_new;

	fp_t* conc_Nb_old;
	fp_t* conc_Nb_new;

	fp_t* phi_del_old;
	fp_t* phi_del_new;

	fp_t* phi_lav_old;
	fp_t* phi_lav_new;

	fp_t* conc_Cr_gam;
	fp_t* conc_Cr_del;
	fp_t* conc_Cr_lav;

	fp_t* conc_Nb_gam;
	fp_t* conc_Nb_del;
	fp_t* conc_Nb_lav;
};

/* src/data.cuh:16 -- prints the error string, records it, returns result.
 * (The reference also assert()s; this library does not abort.) */
cudaError_t checkCuda(cudaError_t result);

/* src/data.cuh:21-25 -- allocates the device fields, creates the streams and
 * events, uploads the nm x nm mask (host->mask_lap[0]) and the constants,
 * copies the four *_old host fields.  nm must be 3. */
void init_cuda(struct HostData* host, const int nx, const int ny, const int nm,
               const fp_t* kappa, const fp_t* omega, const fp_t* Lmob,
               const fp_t* D_Cr, const fp_t* D_Nb, struct CudaData* dev);

/* src/data.cuh:30 */
void free_cuda(struct CudaData* dev);

/* src/data.cuh:35 -- copies the four device *_old fields into host *_new. */
void read_out_result(struct CudaData* dev, struct HostData* host, const int nx, const int ny);

/* src/discretization.cuh:34 */
float nTiles(int domain_size, int tile_loc, int mask_size);

/* src/discretization.cuh:39-118.  In the default fused mode the whole step
 * runs inside device_evolution (old -> new, ghost ring mirrored); the stage
 * functions before it are no-ops because nothing observes their outputs in
 * the reference's call sequence (src/main.cpp:289-305).  In compat mode
 * (pfa_set_mode) each stage reproduces its own post-condition. */
void device_fictitious(struct CudaData* dev, const int nx, const int ny, const int nm,
                       const int bx, const int by);
/* Declared and never defined by the reference (its variable-mobility form is
 * disabled); defined here: in compat mode with pfa_set_mobility's variable
 * mobility they compute the flux coefficients and fill their ghost ring,
 * otherwise they return at once. */
void device_mobilities(struct CudaData* dev, const int nx, const int ny, const int nm,
                       const int bx, const int by);
void device_boundaries(struct CudaData* dev, const int nx, const int ny, const int nm,
                       const int bx, const int by);
void fictitious_boundaries(struct CudaData* dev, const int nx, const int ny, const int nm,
                           const int bx, const int by);
void mobility_boundaries(struct CudaData* dev, const int nx, const int ny, const int nm,
                         const int bx, const int by);
void device_laplacian_boundaries(struct CudaData* dev, const int nx, const int ny, const int nm,
                                 const int bx, const int by);
void device_laplacian(struct CudaData* dev, const int nx, const int ny, const int nm,
                      const int bx, const int by, const fp_t dx, const fp_t dy);
void device_evolution(struct CudaData* dev, const int nx, const int ny, const int nm,
                      const int bx, const int by, const fp_t alpha, const fp_t dt);

/* No per-cell generator state to initialise (Philox is counter-based); this
 * resets the nucleation call counter. */
void device_init_prng(struct CudaData* dev, const int nx, const int ny, const int nm,
                      const int bx, const int by);

/* Deterministic two-phase nucleation on the *_new fields: every interior
 * cell decides on the same snapshot with Philox4x32-10 draws keyed by
 * (seed, call counter, cell), then nuclei are painted in ascending cell order,
 * delta before laves.  Like the reference wrapper, the kernel sees
 * (dx*nx, dy*ny, dz) unless pfa_set_nucleation() selects the fixed geometry. */
void device_nucleation(struct CudaData* dev, const int nx, const int ny, const int nm,
                       const int bx, const int by, const fp_t sigma_del, const fp_t sigma_lav,
                       const fp_t unit_a, const fp_t ifce_width, const fp_t dx, const fp_t dy,
                       const fp_t dz, const fp_t dt);

/* Writes conc_Ni and phi on the device and copies the six host arrays. */
void device_dataviz(struct CudaData* dev, struct HostData* host, const int nx, const int ny,
                    const int nm, const int bx, const int by);

#endif
