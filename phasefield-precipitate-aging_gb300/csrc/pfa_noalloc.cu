// pfa_noalloc.cu -- the field summary without any device allocation.
//
// Some callers cannot let a library allocate device memory: a host that
// hands out all device memory from its own pool and forbids allocation after
// start-up, a fixed memory budget shared by many jobs, or a step loop where
// the implicit device synchronisation of cudaMalloc/cudaFree is not allowed.
// pfa_summarize_fields_noalloc serves them: it computes the same summary as
// pfa_summarize (mean x_Cr, x_Nb and the gamma / delta / laves fractions over
// the interior, src/alloy625.cpp:811-863) from caller-owned device fields and
// writes the five doubles to a caller-owned device buffer.  Its only scratch
// -- one row of five partial sums per grid row -- is the file-scope device
// array below, sized for kNoAllocMaxRows rows (640 KiB; every GPU that loads
// the library holds it until the process exits).
//
// The array is shared by every call: calls whose kernels overlap on the GPU
// (different streams without ordering) race on it.  Nothing needs clearing
// between calls: each call writes every row slot it later reads.
//
// The device address of the array is looked up once per device and kept for
// the life of the process.  cudaDeviceReset unloads the library's device code
// with the context, so the kept address is no longer valid: a process that
// resets a device must not call this entry point on that device afterwards.
#include <mutex>

#include "pfa_device.cuh"
#include "pfa_gb300.h"

namespace pfa {

namespace {

constexpr int kNoAllocMaxRows = 16384;  // interior rows the scratch holds
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_row_sums[kNoAllocMaxRows * 5];

// one CTA per interior row: five compensated sums over the row
__global__ void __launch_bounds__(kThreads) k_row_sums(const double* __restrict__ cr,
                                                       const double* __restrict__ nb,
                                                       const double* __restrict__ pd,
                                                       const double* __restrict__ pl, int nx,
                                                       double* rows) {
  const int y = blockIdx.x + 1;
  double s[5] = {0, 0, 0, 0, 0}, c[5] = {0, 0, 0, 0, 0};
  for (int x = 1 + threadIdx.x; x < nx - 1; x += kThreads) {
    const size_t i = size_t(y) * nx + x;
    const double a = dev::p64(pd[i]), b = dev::p64(pl[i]);
    const double v[5] = {cr[i], nb[i], (1.0 - a) - b, a, b};
#pragma unroll
    for (int k = 0; k < 5; k++) {
      const double yk = v[k] - c[k];
      const double t = s[k] + yk;
      c[k] = (t - s[k]) - yk;
      s[k] = t;
    }
  }
  __shared__ double sh[5][kThreads];
  for (int k = 0; k < 5; k++) sh[k][threadIdx.x] = s[k] - c[k];
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 5; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 5) rows[blockIdx.x * 5 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_rows_total(const double* rows, int nrows, double inv_n, double* out) {
  if (threadIdx.x >= 5) return;
  double s = 0.0, c = 0.0;
  for (int r = 0; r < nrows; r++) {
    const double y = rows[r * 5 + threadIdx.x] - c;
    const double t = s + y;
    c = (t - s) - y;
    s = t;
  }
  out[threadIdx.x] = s * inv_n;
}

std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};  // device address of g_row_sums, per device

}  // namespace

}  // namespace pfa

using namespace pfa;

extern "C" int pfa_summarize_fields_noalloc(const double* conc_Cr, const double* conc_Nb,
                                            const double* phi_del, const double* phi_lav, int nx,
                                            int ny, double* out, void* stream) {
  if (!conc_Cr || !conc_Nb || !phi_del || !phi_lav || !out) {
    set_error(PFA_EINVAL, "pfa_summarize_fields_noalloc: null pointer");
    return PFA_EINVAL;
  }
  if (nx < 3 || ny < 3) {
    set_error(PFA_EINVAL, "pfa_summarize_fields_noalloc: grid smaller than 3 x 3");
    return PFA_EINVAL;
  }
  if (ny - 2 > kNoAllocMaxRows) {
    set_error(PFA_EINVAL,
              "pfa_summarize_fields_noalloc: more than 16384 interior rows (the static "
              "scratch holds one row of partial sums per grid row)");
    return PFA_EINVAL;
  }
  // an error still pending from earlier work on this thread is not this
  // call's: report it as such and leave before launching anything
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    set_error(PFA_ECUDA, "pfa_summarize_fields_noalloc: a CUDA error was pending before the call");
    return PFA_ECUDA;
  }
  int device = 0;
  e = cudaGetDevice(&device);
  if (e != cudaSuccess || device < 0 || device >= kMaxDevices) {
    set_error(PFA_ECUDA, "pfa_summarize_fields_noalloc: no current device");
    return PFA_ECUDA;
  }
  double* rows;
  {
    // set-up, once per device, with that device current: the host-side name
    // of g_row_sums is not a device address; ask the runtime for it
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch[device]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_row_sums);
      if (e != cudaSuccess) {
        set_error(PFA_ECUDA, "pfa_summarize_fields_noalloc: cudaGetSymbolAddress failed");
        return PFA_ECUDA;
      }
      g_scratch[device] = static_cast<double*>(p);
    }
    rows = g_scratch[device];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_row_sums<<<ny - 2, kThreads, 0, s>>>(conc_Cr, conc_Nb, phi_del, phi_lav, nx, rows);
  const double n = double(nx - 2) * double(ny - 2);
  k_rows_total<<<1, 32, 0, s>>>(rows, ny - 2, 1.0 / n, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(PFA_ECUDA, cudaGetErrorString(e));
    return PFA_ECUDA;
  }
  return 0;
}
