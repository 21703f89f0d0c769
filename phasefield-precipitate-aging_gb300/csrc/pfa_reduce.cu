// pfa_reduce.cu -- on-device FP64 field summary of libpfa_gb300.
//
// summarize_fields (src/alloy625.cpp:811-863) averages x_Cr, x_Nb and the
// gamma / delta / laves phase fractions over the grid nodes on the host with
// an OpenMP critical section.  Here the sums run on the device in FP64 with
// Kahan compensation per thread and a fixed two-level order (kSumBlocks
// partial sums, then one block), so repeated calls give identical bits.
#include "pfa_device.cuh"
#include "pfa_reduce.h"

namespace pfa {

using namespace dev;

namespace {

constexpr int kThreads = 256;

struct K5 {
  double s[5], c[5];
  __device__ void add(int k, double v) {
    const double y = v - c[k];
    const double t = s[k] + y;
    c[k] = (t - s[k]) - y;
    s[k] = t;
  }
};

template <class T>
__global__ void __launch_bounds__(kThreads) k_sum_partial(SumArgs a) {
  K5 acc;
  for (int k = 0; k < 5; k++) acc.s[k] = acc.c[k] = 0.0;
  const long long plane = (long long)a.Nx * a.Ny;
  const long long n = plane * a.Nz;
  for (long long t = (long long)blockIdx.x * kThreads + threadIdx.x; t < n;
       t += (long long)gridDim.x * kThreads) {
    const long long z = t / plane, r = t % plane;
    const int y = int(r / a.Nx), x = int(r % a.Nx);
    const size_t cell = a.compact
                            ? (size_t(z) * a.Ny + y) * a.pitch + x
                            : (size_t(a.is3d ? z + 1 : 0) * (a.Ny + 2) + (y + 1)) * a.pitch + (x + 1);
    const size_t i = cell * a.stride;
    double v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = double(static_cast<const T*>(a.f[k])[i]);
    if (a.comp) {  // FP32 form: value = f - c
      const float4 c = a.pack ? cq_unpack(static_cast<const uint2*>(a.comp)[cell])
                              : static_cast<const float4*>(a.comp)[cell];
      v[0] -= double(c.x);
      v[1] -= double(c.y);
      v[2] -= double(c.z);
      v[3] -= double(c.w);
    }
    const double xcr = v[0], xnb = v[1], phd = v[2], phl = v[3];
    const double pd = p64(phd), pl = p64(phl);
    acc.add(0, xcr);
    acc.add(1, xnb);
    acc.add(2, (1.0 - pd) - pl);
    acc.add(3, pd);
    acc.add(4, pl);
  }
  __shared__ double sh[5][kThreads];
  for (int k = 0; k < 5; k++) sh[k][threadIdx.x] = acc.s[k] - acc.c[k];
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 5; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 5) a.partial[blockIdx.x * 5 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_sum_final(const double* partial, int nblocks, double inv_n, double* out) {
  if (threadIdx.x >= 5) return;
  double s = 0.0, c = 0.0;
  for (int b = 0; b < nblocks; b++) {
    const double y = partial[b * 5 + threadIdx.x] - c;
    const double t = s + y;
    c = (t - s) - y;
    s = t;
  }
  out[threadIdx.x] = s * inv_n;
}

}  // namespace

cudaError_t launch_summarize(const SumArgs& a, cudaStream_t s) {
  if (a.is_f32)
    k_sum_partial<float><<<kSumBlocks, kThreads, 0, s>>>(a);
  else
    k_sum_partial<double><<<kSumBlocks, kThreads, 0, s>>>(a);
  const double n = double(a.Nx) * double(a.Ny) * double(a.Nz);
  k_sum_final<<<1, 32, 0, s>>>(a.partial, kSumBlocks, 1.0 / n, a.out);
  return cudaGetLastError();
}

}  // namespace pfa
