// pfa_nucleation.h -- nucleation kernels of libpfa_gb300.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace pfa {

constexpr int kNucCap = 1 << 14;  // events per nucleation call (scratch capacity)
constexpr int kNucIdxBits = 14;   // low key bits carrying the event index
constexpr double kNucMaxScan = 64.0;    // largest neighbourhood scan radius (cells)
constexpr double kNucMaxRadius = 256.0; // largest nucleus radius painted (cells)

struct NucEvent {
  long long cell;  // reference linear index nx * y + x (halo layout)
  int mask;        // bit 0 delta, bit 1 laves
  int pad;
  double xcr, xnb; // composition before painting
  double r[2];     // nucleus radius in cells (delta, laves)
};

// bytes of a nucleation handle's event buffer: kNucCap events and their sort keys
constexpr size_t nucleation_event_bytes() {
  return (sizeof(NucEvent) + sizeof(unsigned long long)) * size_t(kNucCap);
}

struct NucArgs {
  void* f[4];          // x_Cr, x_Nb, phi_del, phi_lav (halo layout, row pitch `pitch`)
  void* comp;          // FP32 form: compensation records (value = f - c; set where
                       // painted), packed 16-bit counts (pack) or float4; else nullptr
  int pack;
  int is_f32;
  int compact;         // FP32 form layout: interior rows only (ghost cells read
                       // as their mirrored interior cell, never painted)
  int stride;          // elements between consecutive cells of f[k] (4 for FP32 records)
  int Nx, Ny, pitch;
  int Nz, is3d;        // 3D grids: Nz interior planes (halo layout: (Nz+2) planes)
  double sigma[2];
  double dx;           // kernel spacing (the reference passes dx * nx here)
  double dV, Vatom, n_gam, dt, R_scan;
  double ln_dtdV, ln_ngam;
  float lnK[2], lnC1[2], C2[2];  // per-phase constants of the FP32 screen (ln_z_tier1/2)
  int scan_lo, scan_hi;  // scan offsets i in [scan_lo, scan_hi) (from R_scan)
  int scan_r2;           // largest integer below R_scan^2
  uint64_t seed;
  unsigned long long* call_ptr;  // scratch: nucleation call counter (Philox counter word)
  NucEvent* events;    // scratch: kNucCap events, then kNucCap sort keys
  unsigned long long* keys;  // = (unsigned long long*)(events + kNucCap)
  unsigned* count;     // scratch: [0] events, [1] cells listed for the FP64 decision
  int* status;         // scratch: 1 = overflow
  int cap;
  long long* cand;     // scratch: cells the FP32 screen left to the FP64 decision
  int cand_cap;        // nucleation_cand_cap(cells)
};

// Length of the FP64-decision list: a quarter of the cells (at least 1024,
// at most 2^24); cells beyond it are decided in place, with the same result.
inline int nucleation_cand_cap(size_t cells) {
  const size_t q = cells / 4;
  return int(q < 1024 ? 1024 : (q > (size_t(1) << 24) ? (size_t(1) << 24) : q));
}

// Device scratch of a nucleation handle: events, counters, status, list.
inline size_t nucleation_scratch_bytes(size_t cells) {
  return nucleation_event_bytes() + 2 * sizeof(unsigned) + sizeof(int) +
         sizeof(unsigned long long) + sizeof(long long) * size_t(nucleation_cand_cap(cells));
}

cudaError_t launch_nucleation(const NucArgs& a, cudaStream_t s);
// Host part of a call: validates the spacing (dx sets the scan and nucleus
// radii in cells, dV = dx dy dz), time step and lattice constant and fills
// the derived fields of `a` (a.sigma, a.is3d, a.Nz set before); returns an
// error message or nullptr.
const char* nucleation_constants(NucArgs& a, double dx, double dy, double dz, double dt,
                                 double unit_a);
cudaError_t nucleation_setup();
cudaError_t launch_philox_block(const void* ctr, uint64_t key, void* out, int n, cudaStream_t s);
cudaError_t launch_split_block(const double* in, float* hi, float* c, int n, cudaStream_t s);

}  // namespace pfa
