// pfa_energy.cu -- on-device free energy of a grid (FP64).
//
// summarize_energy (src/alloy625.cpp:865-919) with gibbs (:752-786) and
// maskedgradient (:788-807), which the reference evaluates on the host at
// every output step: per interior node
//   chem = dV (pGam g_gam(x^gam) + pDel g_del(x^del) + pLav g_lav(x^lav)
//              + sum_i omega_i phi_i^2 (1 - phi_i)^2 + 2 Omega phi_del^2 phi_lav^2)
//   grad = dV sum_i kappa_i |grad phi_i|^2  (central differences over the
//          ghost ring at the edges)
// and the total of chem + grad.  The reference's atomic accumulation has no
// fixed order; here each of kSumBlocks blocks sums a fixed set of nodes in a
// fixed order and one block adds the partials, so the total is reproducible.
#include "pfa_device.cuh"
#include "pfa_reduce.h"

namespace pfa {

using namespace dev;

namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_energy_partial(EnergyArgs a) {
  const size_t nx = size_t(a.Nx) + 2, ny = size_t(a.Ny) + 2;
  const size_t plane = nx * ny;
  const size_t cells = size_t(a.Nx) * a.Ny * (a.is3d ? a.Nz : 1);
  const double dV = a.dxyz[0] * a.dxyz[1] * (a.is3d ? a.dxyz[2] : 1.0);
  const double w[3] = {1.0 / (2.0 * a.dxyz[0]), 1.0 / (2.0 * a.dxyz[1]),
                       1.0 / (2.0 * a.dxyz[2])};
  double acc = 0.0;
  for (size_t c = size_t(blockIdx.x) * kThreads + threadIdx.x; c < cells;
       c += size_t(gridDim.x) * kThreads) {
    const size_t x = c % a.Nx + 1;
    const size_t rest = c / a.Nx;
    const size_t y = rest % a.Ny + 1;
    const size_t z = a.is3d ? rest / a.Ny + 1 : 0;
    const size_t i = z * plane + y * nx + x;
    const double X = a.f[0][i], Y = a.f[1][i];
    const double phi[2] = {a.f[2][i], a.f[3][i]};
    const double pD = p64(phi[0]), pL = p64(phi[1]);
    const double pG = 1.0 - pD - pL;
    Poly64 m;
    poly64(pD, pG, pL, m);
    double g = pG * g64<0>(fict64<0, 0>(X, Y, m), fict64<0, 1>(X, Y, m));
    g += pD * g64<1>(fict64<1, 0>(X, Y, m), fict64<1, 1>(X, Y, m));
    g += pL * g64<2>(fict64<2, 0>(X, Y, m), fict64<2, 1>(X, Y, m));
    const double sq[2] = {phi[0] * phi[0], phi[1] * phi[1]};
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const double u = 1.0 - phi[k];
      g += a.omega[k] * sq[k] * (u * u);
    }
    g += 2.0 * a.Omega * sq[0] * sq[1];
    double ge = 0.0;
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const double* p = a.f[2 + k];
      const double gx = w[0] * (p[i + 1] - p[i - 1]);
      const double gy = w[1] * (p[i + nx] - p[i - nx]);
      double s = gx * gx + gy * gy;
      if (a.is3d) {
        const double gz = w[2] * (p[i + plane] - p[i - plane]);
        s += gz * gz;
      }
      ge += a.kappa[k] * s;
    }
    const double ce = g * dV, ee = ge * dV;
    if (a.chem) a.chem[i] = ce;
    if (a.grad) a.grad[i] = ee;
    acc += ce + ee;
  }
  __shared__ double sh[kThreads];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) a.partial[blockIdx.x] = sh[0];
}

__global__ void k_energy_total(const double* partial, int n, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int k = 0; k < n; k++) s += partial[k];
  *out = s;
}

}  // namespace

cudaError_t launch_energy(const EnergyArgs& a, cudaStream_t s) {
  k_energy_partial<<<kSumBlocks, kThreads, 0, s>>>(a);
  k_energy_total<<<1, 32, 0, s>>>(a.partial, kSumBlocks, a.out);
  return cudaGetLastError();
}

}  // namespace pfa
