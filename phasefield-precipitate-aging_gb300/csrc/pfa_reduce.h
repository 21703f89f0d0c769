// pfa_reduce.h -- field summary kernels of libpfa_gb300.
#pragma once

#include <cuda_runtime.h>

namespace pfa {

constexpr int kSumBlocks = 256;  // fixed partial-sum count (deterministic order)

struct SumArgs {
  const void* f[4];   // fields in the halo layout
  const void* comp;   // FP32 form: compensation records (value = f - c), or nullptr
  int pack;           // comp holds packed 16-bit counts (else float4)
  int is_f32, is3d;
  int compact;        // interior-only rows (FP32 form) instead of the ghost-ring layout
  int stride;         // elements between consecutive cells of f (4 for FP32 records)
  int Nx, Ny, Nz, pitch;
  double* partial;    // scratch: kSumBlocks * 5 doubles
  double* out;        // 5 doubles (device)
};

cudaError_t launch_summarize(const SumArgs& a, cudaStream_t s);

// Free energy of FP64 fields in the ghost-ring layout (pfa_energy.cu).
struct EnergyArgs {
  const double* f[4];
  int Nx, Ny, Nz, is3d;
  double dxyz[3];
  double kappa[2], omega[2], Omega;
  double* chem;       // per-node chemical energy (ghost-ring layout) or nullptr
  double* grad;       // per-node gradient energy or nullptr
  double* partial;    // scratch: kSumBlocks doubles
  double* out;        // 1 double (device)
};

cudaError_t launch_energy(const EnergyArgs& a, cudaStream_t s);

}  // namespace pfa
