// pfa_kernels.h -- kernel argument blocks and launchers of libpfa_gb300.
#pragma once

#include <cstdint>

#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>

#include "pfa_internal.h"

struct pfa_ic_recipe;  // pfa_gb300.h

namespace pfa {

// Arguments of one fused 2D step (passed by value to the kernel).
struct Step2DArgs {
  const void* in[4];    // FP64: x_Cr, x_Nb, phi_del, phi_lav; FP32 form: in[0] = A
                        // records, in[1] = B (compensation) records
  void* out[4];
  int Nx, Ny, pitch;    // interior size and row pitch (elements)
  int write_halo;       // also write the mirrored ghost ring
  int varmob;           // FP64: variable-mobility Cahn-Hilliard (5-point mask)
  int nine;             // 3x3 mask has non-zero corners
  int full_comp;        // FP32 form: compensations as FP32 (16-byte B records)
                        // instead of packed 16-bit counts (8-byte B records)
  ModelConst m;
  double mask9[9];      // full 3x3 mask, row-major (rows y-1..y+1)
  FastCoef k;
  float dtD[2][2];      // dt * D
  float dtL[2];         // dt * L
  float om2[2];         // 2 omega
  float alpha2;         // 2 alpha
  float kap[2];         // kappa
  float idx2f[2];       // 1/dx^2, 1/dy^2
  float lap9[4];        // FP32 form, 9-point mask (symmetric): left / right weight,
                        // upper / lower weight, corner weight, sum of the nine
  float lap9xe[2];      // the sum of the nine weights times xe_gamma (Cr, Nb)
  float vm_pre[3];      // FP32 form, variable mobility: the mobility prefactors
                        // (Nb, Cr, Ni) times dt / (2 dx^2)
  float vm_qy;          // and the weight of the y faces, (1/dy^2) / (1/dx^2)
  int rows;             // FP32 form: rows per warp segment (set by the launcher)
};

// Layout conversion between FP64 reference fields (ghost ring, pitch64) and
// the FP32 form's records (interior only, rows of pitch32 records):
// A = {x_Cr, x_Nb, phi_del, phi_lav} per cell, B = the four Kahan
// compensations, packed 16-bit counts (pack) or FP32.
struct ConvArgs {
  double* f64[4];
  float* A;
  void* B;
  int pack;
  int Nx, Ny, pitch64, pitch32;
  int y0, y1;  // interior rows converted, [y0, y1); y1 = 0: all rows
};

// Arguments of the reference's per-stage kernels (compat mode).
struct StageArgs {
  double* f[4];         // fields the stage reads (old) or fills
  double* o[4];         // fields the stage writes (new / Laplacians)
  double* gam[2];       // fictitious gamma compositions
  double* del[2];       // fictitious delta compositions
  double* lav[2];       // fictitious laves compositions
  int nx, ny;           // full array extent including the ghost ring
  ModelConst m;
  double mask9[9];
  // variable-mobility Cahn-Hilliard: the 16 coefficient arrays (Cr row, Nb
  // row; see dev::mobility64), the spacing of the divergence, and whether
  // the evolution takes the divergence (x + dt div) instead of D lap x^gamma
  double* mob[16];
  double dxy[2];
  int varmob;
};

// A batch of 2D grids in the FP32 form (packed compensations) stepped by one
// launch.  Per grid: record buffers of both parities; per unit of work: one
// warp strip (30 columns) over a row segment of one grid.
struct BatchGrid {
  float4* A[2];   // {x_Cr, x_Nb, phi_del, phi_lav} records, parity 0 / 1
  uint2* B[2];    // packed Kahan compensations
  int Nx, Ny, pitch, pad;
};
struct BatchUnit {
  int grid, x0, y0, y1;
};
struct BatchArgs {
  const BatchGrid* grid;
  const BatchUnit* unit;
  int* counter;   // unit counters of parity 0 / 1, then the unit count
  int units;      // one-warp-per-unit mode: units of this launch
  int parity;     // records are read from parity, written to parity ^ 1
  int persistent;
};

cudaError_t launch_step2d_f64(const Step2DArgs& a, cudaStream_t s);
cudaError_t launch_step2d_f32(const Step2DArgs& a, cudaStream_t s);
cudaError_t prepare_step2d_f32();
// ctas: CTAs of a persistent launch (b.persistent), else one warp per unit
cudaError_t launch_batch_f32(const Step2DArgs& a, const BatchArgs& b, int ctas, cudaStream_t s);
int batch_resident_ctas();   // CTAs of k_batch_f32 resident on the device at once
int batch_warps_per_cta();
int batch_strip_cols();
cudaError_t launch_import_f32(const ConvArgs& a, cudaStream_t s);

// initial conditions from a recipe (pfa_ic.cu): validation (message or
// nullptr) and the fill of four FP64 fields in the reference layout
const char* ic_check(const ::pfa_ic_recipe* r);
cudaError_t launch_ic_fill(const ::pfa_ic_recipe& r, double* const f[4], cudaStream_t s);
cudaError_t launch_export_f32(const ConvArgs& a, cudaStream_t s);

// Arguments of one 3D step (pfa_step3d.cu).  F64: in/out = four ghost-ring
// arrays ((Nz+2) x (Ny+2) x pitch, pitch = Nx + 2); FP32 form: in[0]/out[0]
// = float4 A records, in[1]/out[1] = packed compensation records (uint2),
// Nz x Ny x pitch.
struct Step3DArgs {
  const void* in[4];
  void* out[4];
  int Nx, Ny, Nz, pitch;
  int zrows;            // z planes per segment (set by the launcher)
  ModelConst m;         // m.idx2 = 1/dx^2, 1/dy^2, 1/dz^2
  FastCoef k;
  float dtD[2][2], dtL[2], om2[2], alpha2, kap[2], idx2f[3];
  int* status;          // FP32 form: set to 3 when a staging wait gave up (may be null)
  int skip_plane;       // tests only: CTA (0, 0, 0) neither arms nor issues the
                        // copies of this interior plane (>= 0), so its wait runs
                        // out; negative: none (plane -1 is the ring's lower halo)
};

// TMA descriptors of one FP32-form record pair (A: the float4 records as an
// FP32 tensor of (4 Nx, Ny, Nz); B: the packed compensations as a uint32
// tensor of (2 Nx, Ny, Nz); rows pitch records apart)
struct Tma3 {
  CUtensorMap a, b;
};

struct Conv3DArgs {
  double* f64[4];  // ghost-ring layout
  float* A;        // float4 records
  void* B;         // packed compensation records (uint2)
  int Nx, Ny, Nz, pitch32;
};

cudaError_t prepare_step3d();
cudaError_t encode_step3d_maps(Tma3* t, const void* A, const void* B, int Nx, int Ny, int Nz,
                               int pitch);
// t: the maps of a.in[0] / a.in[1] (FP32 form; unused for FP64)
cudaError_t launch_step3d(Step3DArgs a, bool f64, const Tma3* t, cudaStream_t s);
cudaError_t launch_import3d(const Conv3DArgs& a, cudaStream_t s);
cudaError_t launch_export3d(const Conv3DArgs& a, cudaStream_t s);

// compat-mode stages (pfa_stages.cu)
cudaError_t launch_bc(double* f, int nx, int ny, cudaStream_t s);
cudaError_t launch_fictitious(const StageArgs& a, cudaStream_t s);
cudaError_t launch_convolution(const double* in, double* out, int nx, int ny,
                               const double* mask9, cudaStream_t s);
cudaError_t launch_evolution(const StageArgs& a, cudaStream_t s);
// variable mobility: the 16 coefficients at every cell (a.gam/del/lav hold the
// fictitious compositions), and the divergences of Cr and Nb into a.o[0], a.o[1]
cudaError_t launch_mobility(const StageArgs& a, cudaStream_t s);
cudaError_t launch_chem_convolution(const StageArgs& a, cudaStream_t s);
// the fused FP64 variable-mobility step's one-time set-up (shared memory)
cudaError_t prepare_step2d_f64();
cudaError_t launch_dataviz(const double* cr, const double* nb, const double* pd,
                           const double* pl, double* ni, double* phi, int nx, int ny,
                           cudaStream_t s);

}  // namespace pfa
