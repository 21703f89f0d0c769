// pfa_stages.cu -- per-stage kernels behind the reference's stage functions.
//
// In compat mode each reference host function keeps its own post-condition:
//   device_boundaries / fictitious_boundaries / device_laplacian_boundaries
//       -> zero-flux ghost fill (boundary_kernel, src/discretization.cu:360-394)
//   device_fictitious -> gamma, delta, laves compositions (:50-126)
//   device_laplacian  -> 3x3 mask convolution into the *_new arrays (:550-603)
//   device_evolution  -> CH + AC from those Laplacians (:843-1020)
//   device_dataviz    -> x_Ni and p(phi_del) + p(phi_lav) (:1211-1229)
// and, with the variable-mobility Cahn-Hilliard, the reference's disabled
//   device_mobilities -> the 16 flux coefficients (:175-358)
//   device_laplacian  -> chemical_convolution_Cr/Nb (:618-778) for x_Cr, x_Nb
//   device_evolution  -> x + dt div (the commented composition_kernel, :848-856)
// The fused path (pfa_step2d.cu) is the production form; these kernels let a
// caller observe every intermediate the reference exposes.
#include "pfa_device.cuh"
#include "pfa_kernels.h"

namespace pfa {

using namespace dev;

namespace {

// Ghost cell <- nearest interior cell (corners take the diagonal cell; the
// reference fills the four sides concurrently, leaving its corners racy).
__global__ void k_bc(double* f, int nx, int ny) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  int hx, hy;
  if (t < nx) {
    hx = t;
    hy = 0;
  } else if (t < 2 * nx) {
    hx = t - nx;
    hy = ny - 1;
  } else if (t < 2 * nx + ny) {
    hx = 0;
    hy = t - 2 * nx;
  } else if (t < 2 * nx + 2 * ny) {
    hx = nx - 1;
    hy = t - 2 * nx - ny;
  } else {
    return;
  }
  const int sx = hx < 1 ? 1 : (hx > nx - 2 ? nx - 2 : hx);
  const int sy = hy < 1 ? 1 : (hy > ny - 2 ? ny - 2 : hy);
  f[size_t(hy) * nx + hx] = f[size_t(sy) * nx + sx];
}

__global__ void k_fictitious(StageArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.nx || y >= a.ny) return;
  const size_t i = size_t(y) * a.nx + x;
  const double X = a.f[0][i], Y = a.f[1][i];
  const double pD = p64(a.f[2][i]), pL = p64(a.f[3][i]), pG = 1.0 - pD - pL;
  Poly64 m;
  poly64(pD, pG, pL, m);
  a.gam[0][i] = fict64<0, 0>(X, Y, m);
  a.gam[1][i] = fict64<0, 1>(X, Y, m);
  if (a.del[0]) {
    a.del[0][i] = fict64<1, 0>(X, Y, m);
    a.del[1][i] = fict64<1, 1>(X, Y, m);
  }
  if (a.lav[0]) {
    a.lav[0][i] = fict64<2, 0>(X, Y, m);
    a.lav[1][i] = fict64<2, 1>(X, Y, m);
  }
}

struct Mask9 {
  double m[9];
};

// Interior cells only; the ghost ring is left for the boundary stage.
__global__ void k_convolution(const double* __restrict__ in, double* __restrict__ out, int nx,
                              int ny, Mask9 mk) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (x > nx - 2 || y > ny - 2) return;
  double v = 0.0;
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int i = 0; i < 3; i++) v += mk.m[j * 3 + i] * in[size_t(y + j - 1) * nx + (x + i - 1)];
  out[size_t(y) * nx + x] = v;
}

// Every cell, ghost ring included, as the reference's update kernels do.
__global__ void k_evolution(StageArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.nx || y >= a.ny) return;
  const size_t i = size_t(y) * a.nx + x;
  const ModelConst& M = a.m;
  const double X = a.f[0][i], Y = a.f[1][i], phd = a.f[2][i], phl = a.f[3][i];
  const double lapCr = a.o[0][i], lapNb = a.o[1][i], lapD = a.o[2][i], lapL = a.o[3][i];
  if (a.varmob) {  // lapCr, lapNb hold the divergences
    a.o[0][i] = X + M.dt * lapCr;
    a.o[1][i] = Y + M.dt * lapNb;
  } else {
    a.o[0][i] = X + M.dt * (M.D[0][0] * lapCr + M.D[0][1] * lapNb);
    a.o[1][i] = Y + M.dt * (M.D[1][0] * lapCr + M.D[1][1] * lapNb);
  }
  const double pD = p64(phd), pL = p64(phl), pG = 1.0 - pD - pL;
  Poly64 m;
  poly64(pD, pG, pL, m);
  const double gam_Cr = fict64<0, 0>(X, Y, m), gam_Nb = fict64<0, 1>(X, Y, m);
  const double gam_nrg = g64<0>(gam_Cr, gam_Nb);
  const double dgGdxCr = dg64<0>(gam_Cr, gam_Nb), dgGdxNb = dg64<1>(gam_Cr, gam_Nb);
  {
    const double del_Cr = fict64<1, 0>(X, Y, m), del_Nb = fict64<1, 1>(X, Y, m);
    const double gp = gam_nrg - g64<1>(del_Cr, del_Nb) - dgGdxCr * (gam_Cr - del_Cr) -
                      dgGdxNb * (gam_Nb - del_Nb);
    const double dF = -pp64(phd) * gp + 2.0 * M.omega[0] * phd * (phd - 1.0) * (2.0 * phd - 1.0) +
                      2.0 * M.alpha * phd * phl * phl - M.kappa[0] * lapD;
    a.o[2][i] = phd - M.dt * M.L[0] * dF;
  }
  {
    const double lav_Cr = fict64<2, 0>(X, Y, m), lav_Nb = fict64<2, 1>(X, Y, m);
    const double gp = gam_nrg - g64<2>(lav_Cr, lav_Nb) - dgGdxCr * (gam_Cr - lav_Cr) -
                      dgGdxNb * (gam_Nb - lav_Nb);
    const double dF = -pp64(phl) * gp + 2.0 * M.omega[1] * phl * (phl - 1.0) * (2.0 * phl - 1.0) +
                      2.0 * M.alpha * phl * phd * phd - M.kappa[1] * lapL;
    a.o[3][i] = phl - M.dt * M.L[1] * dF;
  }
}

// Every cell, ghost ring included (mobility_Cr/Nb_kernel run over the whole
// array); the fictitious compositions come from k_fictitious.
__global__ void k_mobility(StageArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.nx || y >= a.ny) return;
  const size_t i = size_t(y) * a.nx + x;
  const double X = a.f[0][i], Y = a.f[1][i], phd = a.f[2][i], phl = a.f[3][i];
  const double pD = p64(phd), pL = p64(phl), pG = 1.0 - pD - pL;
  const double xg[2] = {a.gam[0][i], a.gam[1][i]};
  const double xd[2] = {a.del[0][i], a.del[1][i]};
  const double xl[2] = {a.lav[0][i], a.lav[1][i]};
  double o[16];
  mobility64(X, Y, phd, phl, pD, pG, pL, xg, xd, xl, o);
#pragma unroll
  for (int k = 0; k < 16; k++) a.mob[k][i] = o[k];
}

// chemical_convolution_Cr_kernel / _Nb_kernel at the interior cells (the
// ghost ring is left to the boundary stage): for the coefficient / field
// pairs of terms 1-6 the differences along x and along y, for terms 7-8
// along x only, in the reference's order.
__global__ void k_chem_convolution(StageArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (x > a.nx - 2 || y > a.ny - 2) return;
  const size_t mid = size_t(y) * a.nx + x, lft = mid - 1, rgt = mid + 1, bot = mid - a.nx,
               top = mid + a.nx;
  const double r2x = 1.0 / (2.0 * a.dxy[0] * a.dxy[0]), r2y = 1.0 / (2.0 * a.dxy[1] * a.dxy[1]);
  const double* c[6] = {a.gam[0], a.gam[1], a.del[0], a.del[1], a.lav[0], a.lav[1]};
#pragma unroll
  for (int k = 0; k < 2; k++) {
    double* const* mob = a.mob + 8 * k;
    double div = 0.0;
#pragma unroll
    for (int t = 0; t < 6; t++) {
      const double* D = mob[t];
      div += dlap64(D[lft], D[mid], D[rgt], c[t][lft], c[t][mid], c[t][rgt], r2x);
      div += dlap64(D[bot], D[mid], D[top], c[t][bot], c[t][mid], c[t][top], r2y);
    }
    div += dlap64(mob[6][lft], mob[6][mid], mob[6][rgt], a.f[2][lft], a.f[2][mid], a.f[2][rgt], r2x);
    div += dlap64(mob[7][lft], mob[7][mid], mob[7][rgt], a.f[3][lft], a.f[3][mid], a.f[3][rgt], r2x);
    a.o[k][mid] = div;
  }
}

__global__ void k_dataviz(const double* cr, const double* nb, const double* pd, const double* pl,
                          double* ni, double* phi, int nx, int ny) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= nx || y >= ny) return;
  const size_t i = size_t(y) * nx + x;
  ni[i] = 1.0 - cr[i] - nb[i];
  phi[i] = p64(pd[i]) + p64(pl[i]);
}

dim3 grid2(int nx, int ny) { return dim3((nx + 31) / 32, (ny + 7) / 8); }

}  // namespace

cudaError_t launch_bc(double* f, int nx, int ny, cudaStream_t s) {
  const int n = 2 * nx + 2 * ny;
  k_bc<<<(n + 255) / 256, 256, 0, s>>>(f, nx, ny);
  return cudaGetLastError();
}

cudaError_t launch_fictitious(const StageArgs& a, cudaStream_t s) {
  k_fictitious<<<grid2(a.nx, a.ny), dim3(32, 8), 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_convolution(const double* in, double* out, int nx, int ny, const double* mask9,
                               cudaStream_t s) {
  Mask9 mk;
  for (int k = 0; k < 9; k++) mk.m[k] = mask9[k];
  k_convolution<<<grid2(nx - 2, ny - 2), dim3(32, 8), 0, s>>>(in, out, nx, ny, mk);
  return cudaGetLastError();
}

cudaError_t launch_evolution(const StageArgs& a, cudaStream_t s) {
  k_evolution<<<grid2(a.nx, a.ny), dim3(32, 8), 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_mobility(const StageArgs& a, cudaStream_t s) {
  k_mobility<<<grid2(a.nx, a.ny), dim3(32, 8), 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_chem_convolution(const StageArgs& a, cudaStream_t s) {
  k_chem_convolution<<<grid2(a.nx - 2, a.ny - 2), dim3(32, 8), 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_dataviz(const double* cr, const double* nb, const double* pd, const double* pl,
                           double* ni, double* phi, int nx, int ny, cudaStream_t s) {
  k_dataviz<<<grid2(nx, ny), dim3(32, 8), 0, s>>>(cr, nb, pd, pl, ni, phi, nx, ny);
  return cudaGetLastError();
}

}  // namespace pfa
