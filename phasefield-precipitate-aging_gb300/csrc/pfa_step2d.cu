// pfa_step2d.cu -- 2D step kernels of libpfa_gb300 (sm_103a).
//
// One fused kernel per explicit Euler step replaces the reference's 29
// launches (src/main.cpp:289-305): zero-flux boundary fill, fictitious
// gamma compositions (src/discretization.cu:50-74), 5- or 9-point mask
// convolution (:550-603), Cahn-Hilliard (:843-886) and Allen-Cahn (:888-980).
// Each CTA stages one tile plus its one-cell halo in shared memory, computes
// p(phi) and x^gamma once per staged cell, then the Laplacians and both
// updates for its interior cells.  Domain edges are handled by clamped
// (mirrored) indexing, which is what the reference's halo fill produces.
//
// Layout: the reference's, (Ny + 2) rows of pitch elements with a one-cell
// ghost ring, interior cell (x, y) at (y + 1) * pitch + x + 1.  The FP32
// precision form has its own kernel and layout (pfa_step2d_f32.cu).
#include <cstdint>

#include "pfa_device.cuh"
#include "pfa_kernels.h"

namespace pfa {

using namespace dev;

namespace {

constexpr int kTX = 32;   // tile width (one warp)
constexpr int kTY = 16;   // tile height
constexpr int kBY = 8;    // thread rows per CTA
constexpr int kEX = kTX + 2;
constexpr int kEY = kTY + 2;

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Write a value to interior cell (gx, gy) and, for cells on the domain edge,
// to the ghost cells that mirror it (corners take the diagonal value).
template <class T>
__device__ __forceinline__ void store_with_halo(T* f, int pitch, int gx, int gy, int Nx, int Ny,
                                                T v, bool halo) {
  const size_t row = size_t(gy + 1) * pitch;
  f[row + gx + 1] = v;
  if (!halo) return;
  const bool l = gx == 0, r = gx == Nx - 1, b = gy == 0, t = gy == Ny - 1;
  if (l) f[row] = v;
  if (r) f[row + Nx + 1] = v;
  if (b) {
    f[gx + 1] = v;
    if (l) f[0] = v;
    if (r) f[Nx + 1] = v;
  }
  if (t) {
    const size_t top = size_t(Ny + 1) * pitch;
    f[top + gx + 1] = v;
    if (l) f[top] = v;
    if (r) f[top + Nx + 1] = v;
  }
}

// ---------------------------------------------------------------------------
// Plain FP64 fused step (faithful to the reference's formulas).
// NINE: the mask has non-zero corners (9-point stencil, src/mesh.cpp:198-213).
template <bool NINE>
__global__ void __launch_bounds__(kTX* kBY) k_step2d_f64(Step2DArgs a) {
  __shared__ double s_phd[kEY][kEX], s_phl[kEY][kEX], s_gcr[kEY][kEX], s_gnb[kEY][kEX];
  __shared__ double s_pd[kEY][kEX], s_pl[kEY][kEX], s_rden[kEY][kEX];
  const double* __restrict__ icr = static_cast<const double*>(a.in[0]);
  const double* __restrict__ inb = static_cast<const double*>(a.in[1]);
  const double* __restrict__ ipd = static_cast<const double*>(a.in[2]);
  const double* __restrict__ ipl = static_cast<const double*>(a.in[3]);
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
  const int tid = threadIdx.y * kTX + threadIdx.x;

  for (int e = tid; e < kEX * kEY; e += kTX * kBY) {
    const int ex = e % kEX, ey = e / kEX;
    const int gx = clampi(x0 + ex - 1, 0, a.Nx - 1);
    const int gy = clampi(y0 + ey - 1, 0, a.Ny - 1);
    const size_t i = size_t(gy + 1) * a.pitch + gx + 1;
    const double X = icr[i], Y = inb[i], phd = ipd[i], phl = ipl[i];
    const double pD = p64(phd), pL = p64(phl), pG = 1.0 - pD - pL;
    Poly64 m;
    poly64(pD, pG, pL, m);
    s_phd[ey][ex] = phd;
    s_phl[ey][ex] = phl;
    s_gcr[ey][ex] = fict64<0, 0>(X, Y, m);
    s_gnb[ey][ex] = fict64<0, 1>(X, Y, m);
    s_pd[ey][ex] = pD;
    s_pl[ey][ex] = pL;
    s_rden[ey][ex] = m.rden;
  }
  __syncthreads();

  const ModelConst& M = a.m;
  for (int r = threadIdx.y; r < kTY; r += kBY) {
    const int gx = x0 + threadIdx.x, gy = y0 + r;
    if (gx >= a.Nx || gy >= a.Ny) continue;
    const int ex = threadIdx.x + 1, ey = r + 1;
    // Mask convolution in the reference's order (rows j = y-1..y+1, columns
    // i = x-1..x+1, value += mask * tile, contracted to FMA); zero mask
    // entries are exact no-ops there and are skipped for the 5-point mask.
    auto lap = [&](double (*s)[kEX]) {
      double v;
      if (NINE) {
        v = a.mask9[0] * s[ey - 1][ex - 1];
        v = fma(a.mask9[1], s[ey - 1][ex], v);
        v = fma(a.mask9[2], s[ey - 1][ex + 1], v);
        v = fma(a.mask9[3], s[ey][ex - 1], v);
        v = fma(a.mask9[4], s[ey][ex], v);
        v = fma(a.mask9[5], s[ey][ex + 1], v);
        v = fma(a.mask9[6], s[ey + 1][ex - 1], v);
        v = fma(a.mask9[7], s[ey + 1][ex], v);
        v = fma(a.mask9[8], s[ey + 1][ex + 1], v);
      } else {
        v = M.mask[0] * s[ey - 1][ex];
        v = fma(M.mask[1], s[ey][ex - 1], v);
        v = fma(M.mask[2], s[ey][ex], v);
        v = fma(M.mask[3], s[ey][ex + 1], v);
        v = fma(M.mask[4], s[ey + 1][ex], v);
      }
      return v;
    };
    const double lapCr = lap(s_gcr), lapNb = lap(s_gnb), lapD = lap(s_phd), lapL = lap(s_phl);
    const size_t i = size_t(gy + 1) * a.pitch + gx + 1;
    const double X = icr[i], Y = inb[i];
    const double phd = s_phd[ey][ex], phl = s_phl[ey][ex];

    // Cahn-Hilliard, composition_kernel src/discretization.cu:843-865
    const double ocr = X + M.dt * (M.D[0][0] * lapCr + M.D[0][1] * lapNb);
    const double onb = Y + M.dt * (M.D[1][0] * lapCr + M.D[1][1] * lapNb);

    // Allen-Cahn, src/discretization.cu:888-980
    Poly64 m;
    m.lin[0] = s_pd[ey][ex];
    m.lin[2] = s_pl[ey][ex];
    m.lin[1] = 1.0 - m.lin[0] - m.lin[2];
    m.mono[0] = m.lin[0] * m.lin[0];
    m.mono[1] = m.lin[0] * m.lin[1];
    m.mono[2] = m.lin[0] * m.lin[2];
    m.mono[3] = m.lin[1] * m.lin[1];
    m.mono[4] = m.lin[1] * m.lin[2];
    m.mono[5] = m.lin[2] * m.lin[2];
    m.rden = s_rden[ey][ex];
    const double gam_Cr = s_gcr[ey][ex], gam_Nb = s_gnb[ey][ex];
    const double gam_nrg = g64<0>(gam_Cr, gam_Nb);
    const double dgGdxCr = dg64<0>(gam_Cr, gam_Nb);
    const double dgGdxNb = dg64<1>(gam_Cr, gam_Nb);
    double od, ol;
    {
      const double del_Cr = fict64<1, 0>(X, Y, m), del_Nb = fict64<1, 1>(X, Y, m);
      const double del_nrg = g64<1>(del_Cr, del_Nb);
      const double gp = gam_nrg - del_nrg - dgGdxCr * (gam_Cr - del_Cr) - dgGdxNb * (gam_Nb - del_Nb);
      const double dF = -pp64(phd) * gp + 2.0 * M.omega[0] * phd * (phd - 1.0) * (2.0 * phd - 1.0) +
                        2.0 * M.alpha * phd * phl * phl - M.kappa[0] * lapD;
      od = phd - M.dt * M.L[0] * dF;
    }
    {
      const double lav_Cr = fict64<2, 0>(X, Y, m), lav_Nb = fict64<2, 1>(X, Y, m);
      const double lav_nrg = g64<2>(lav_Cr, lav_Nb);
      const double gp = gam_nrg - lav_nrg - dgGdxCr * (gam_Cr - lav_Cr) - dgGdxNb * (gam_Nb - lav_Nb);
      const double dF = -pp64(phl) * gp + 2.0 * M.omega[1] * phl * (phl - 1.0) * (2.0 * phl - 1.0) +
                        2.0 * M.alpha * phl * phd * phd - M.kappa[1] * lapL;
      ol = phl - M.dt * M.L[1] * dF;
    }
    const bool h = a.write_halo;
    store_with_halo(static_cast<double*>(a.out[0]), a.pitch, gx, gy, a.Nx, a.Ny, ocr, h);
    store_with_halo(static_cast<double*>(a.out[1]), a.pitch, gx, gy, a.Nx, a.Ny, onb, h);
    store_with_halo(static_cast<double*>(a.out[2]), a.pitch, gx, gy, a.Nx, a.Ny, od, h);
    store_with_halo(static_cast<double*>(a.out[3]), a.pitch, gx, gy, a.Nx, a.Ny, ol, h);
  }
}

// ---------------------------------------------------------------------------
// Plain FP64 step with the variable-mobility Cahn-Hilliard (5-point mask):
// the reference's disabled mobility kernels, chemical_convolution_Cr/Nb
// (src/discretization.cu:175-358, 618-778) and the commented update of
// composition_kernel (:848-856), fused.  Each CTA stages its tile and halo:
// per cell the phases, the six fictitious compositions and the 16 flux
// coefficients (dev::mobility64, three FP64 exponentials), then forms the
// divergences (terms 7-8 along x only, as the reference) and the Laplacians
// of the phases, and updates its interior cells.  Staged arrays are laid out
// one after another in dynamic shared memory (kVmArrays x kVmCells doubles).
constexpr int kVmTY = 8;                      // tile height (one row per thread row)
constexpr int kVmCells = kEX * (kVmTY + 2);   // staged cells (tile + halo)
constexpr int kVmArrays = 27;                 // phd phl fict[6] mob[16] pD pL rden
constexpr size_t kVmSmem = sizeof(double) * kVmArrays * kVmCells;

__global__ void __launch_bounds__(kTX* kVmTY) k_step2d_f64_varmob(Step2DArgs a) {
  extern __shared__ double vm[];
  auto S = [&](int k, int ex, int ey) -> double& { return vm[k * kVmCells + ey * kEX + ex]; };
  const double* __restrict__ icr = static_cast<const double*>(a.in[0]);
  const double* __restrict__ inb = static_cast<const double*>(a.in[1]);
  const double* __restrict__ ipd = static_cast<const double*>(a.in[2]);
  const double* __restrict__ ipl = static_cast<const double*>(a.in[3]);
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kVmTY;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  for (int e = tid; e < kVmCells; e += kTX * kVmTY) {
    const int ex = e % kEX, ey = e / kEX;
    const int gx = clampi(x0 + ex - 1, 0, a.Nx - 1);
    const int gy = clampi(y0 + ey - 1, 0, a.Ny - 1);
    const size_t i = size_t(gy + 1) * a.pitch + gx + 1;
    const double X = icr[i], Y = inb[i], phd = ipd[i], phl = ipl[i];
    const double pD = p64(phd), pL = p64(phl), pG = 1.0 - pD - pL;
    Poly64 m;
    poly64(pD, pG, pL, m);
    const double xg[2] = {fict64<0, 0>(X, Y, m), fict64<0, 1>(X, Y, m)};
    const double xd[2] = {fict64<1, 0>(X, Y, m), fict64<1, 1>(X, Y, m)};
    const double xl[2] = {fict64<2, 0>(X, Y, m), fict64<2, 1>(X, Y, m)};
    double mob[16];
    mobility64(X, Y, phd, phl, pD, pG, pL, xg, xd, xl, mob);
    S(0, ex, ey) = phd;
    S(1, ex, ey) = phl;
    S(2, ex, ey) = xg[0];
    S(3, ex, ey) = xg[1];
    S(4, ex, ey) = xd[0];
    S(5, ex, ey) = xd[1];
    S(6, ex, ey) = xl[0];
    S(7, ex, ey) = xl[1];
#pragma unroll
    for (int k = 0; k < 16; k++) S(8 + k, ex, ey) = mob[k];
    S(24, ex, ey) = pD;
    S(25, ex, ey) = pL;
    S(26, ex, ey) = m.rden;
  }
  __syncthreads();

  const ModelConst& M = a.m;
  const int gx = x0 + threadIdx.x, gy = y0 + threadIdx.y;
  if (gx >= a.Nx || gy >= a.Ny) return;
  const int ex = threadIdx.x + 1, ey = threadIdx.y + 1;
  const double r2x = 0.5 * M.idx2[0], r2y = 0.5 * M.idx2[1];  // 1 / (2 d^2)
  double div[2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int mb = 8 + 8 * k;  // this component's coefficients
    double d = 0.0;
#pragma unroll
    for (int t = 0; t < 6; t++) {
      const int D = mb + t, c = 2 + t;
      d += dlap64(S(D, ex - 1, ey), S(D, ex, ey), S(D, ex + 1, ey), S(c, ex - 1, ey), S(c, ex, ey),
                  S(c, ex + 1, ey), r2x);
      d += dlap64(S(D, ex, ey - 1), S(D, ex, ey), S(D, ex, ey + 1), S(c, ex, ey - 1), S(c, ex, ey),
                  S(c, ex, ey + 1), r2y);
    }
    d += dlap64(S(mb + 6, ex - 1, ey), S(mb + 6, ex, ey), S(mb + 6, ex + 1, ey), S(0, ex - 1, ey),
                S(0, ex, ey), S(0, ex + 1, ey), r2x);
    d += dlap64(S(mb + 7, ex - 1, ey), S(mb + 7, ex, ey), S(mb + 7, ex + 1, ey), S(1, ex - 1, ey),
                S(1, ex, ey), S(1, ex + 1, ey), r2x);
    div[k] = d;
  }
  auto lap = [&](int k) {
    double v = M.mask[0] * S(k, ex, ey - 1);
    v = fma(M.mask[1], S(k, ex - 1, ey), v);
    v = fma(M.mask[2], S(k, ex, ey), v);
    v = fma(M.mask[3], S(k, ex + 1, ey), v);
    return fma(M.mask[4], S(k, ex, ey + 1), v);
  };
  const double lapD = lap(0), lapL = lap(1);
  const size_t i = size_t(gy + 1) * a.pitch + gx + 1;
  const double X = icr[i], Y = inb[i];
  const double phd = S(0, ex, ey), phl = S(1, ex, ey);
  const double ocr = X + M.dt * div[0];
  const double onb = Y + M.dt * div[1];
  // Allen-Cahn, src/discretization.cu:888-980, as in k_step2d_f64
  const double gam_Cr = S(2, ex, ey), gam_Nb = S(3, ex, ey);
  const double gam_nrg = g64<0>(gam_Cr, gam_Nb);
  const double dgGdxCr = dg64<0>(gam_Cr, gam_Nb);
  const double dgGdxNb = dg64<1>(gam_Cr, gam_Nb);
  double od, ol;
  {
    const double del_Cr = S(4, ex, ey), del_Nb = S(5, ex, ey);
    const double del_nrg = g64<1>(del_Cr, del_Nb);
    const double gp = gam_nrg - del_nrg - dgGdxCr * (gam_Cr - del_Cr) - dgGdxNb * (gam_Nb - del_Nb);
    const double dF = -pp64(phd) * gp + 2.0 * M.omega[0] * phd * (phd - 1.0) * (2.0 * phd - 1.0) +
                      2.0 * M.alpha * phd * phl * phl - M.kappa[0] * lapD;
    od = phd - M.dt * M.L[0] * dF;
  }
  {
    const double lav_Cr = S(6, ex, ey), lav_Nb = S(7, ex, ey);
    const double lav_nrg = g64<2>(lav_Cr, lav_Nb);
    const double gp = gam_nrg - lav_nrg - dgGdxCr * (gam_Cr - lav_Cr) - dgGdxNb * (gam_Nb - lav_Nb);
    const double dF = -pp64(phl) * gp + 2.0 * M.omega[1] * phl * (phl - 1.0) * (2.0 * phl - 1.0) +
                      2.0 * M.alpha * phl * phd * phd - M.kappa[1] * lapL;
    ol = phl - M.dt * M.L[1] * dF;
  }
  const bool h = a.write_halo;
  store_with_halo(static_cast<double*>(a.out[0]), a.pitch, gx, gy, a.Nx, a.Ny, ocr, h);
  store_with_halo(static_cast<double*>(a.out[1]), a.pitch, gx, gy, a.Nx, a.Ny, onb, h);
  store_with_halo(static_cast<double*>(a.out[2]), a.pitch, gx, gy, a.Nx, a.Ny, od, h);
  store_with_halo(static_cast<double*>(a.out[3]), a.pitch, gx, gy, a.Nx, a.Ny, ol, h);
}

}  // namespace

// ---------------------------------------------------------------------------
cudaError_t prepare_step2d_f64() {
  return cudaFuncSetAttribute(k_step2d_f64_varmob, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              int(kVmSmem));
}

cudaError_t launch_step2d_f64(const Step2DArgs& a, cudaStream_t s) {
  if (a.varmob) {
    if (a.nine) return cudaErrorInvalidValue;
    dim3 grid((a.Nx + kTX - 1) / kTX, (a.Ny + kVmTY - 1) / kVmTY);
    k_step2d_f64_varmob<<<grid, dim3(kTX, kVmTY), kVmSmem, s>>>(a);
    return cudaGetLastError();
  }
  dim3 grid((a.Nx + kTX - 1) / kTX, (a.Ny + kTY - 1) / kTY);
  dim3 block(kTX, kBY);
  if (a.nine)
    k_step2d_f64<true><<<grid, block, 0, s>>>(a);
  else
    k_step2d_f64<false><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pfa
