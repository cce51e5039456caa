// FP64 fused multiply-add throughput of the GPU a handle runs on, measured
// with CUDA events on the handle's stream.  The residual's face and gradient
// kernels are bound by the FP64 pipe, not by HBM (GB300 issues one FP64 warp
// instruction per ~16 SM cycles); this rate is the denominator of their
// roofline fraction.
#include "ics_internal.cuh"

// identical to the definition in ics_api.cu (one handle type for the ABI)
struct ics_handle_s {
  ics::Handle h;
};

namespace ics {

// eight independent FMA chains per thread; m and c arrive at run time so
// the chains cannot be folded, and the result is stored only if it matches
// a value it never takes, which keeps the chains live
__global__ void __launch_bounds__(256) k_dfma_chains(int iters, double m, double c, double never,
                                                     double* __restrict__ out) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-3 * k + 1e-9 * threadIdx.x;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == never) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace ics

using namespace ics;

extern "C" int ics_measure_fp64_rate(ics_handle hh, double* gflops) {
  if (!hh || !gflops) return ICS_ERR_ARG;
  Handle& h = hh->h;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, h.device) != cudaSuccess) return ICS_ERR_CUDA;
  const int blocks = prop.multiProcessorCount * 8, threads = 256, iters = 8192;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double* out = nullptr;
  cudaError_t e = cudaMalloc(&out, (size_t)blocks * threads * sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float ms = 0.0f;
  if (e == cudaSuccess) {
    k_dfma_chains<<<blocks, threads, 0, h.stream>>>(iters / 8, 0.999999999, 1e-9, -1.0, out);  // warm-up
    cudaEventRecord(e0, h.stream);
    k_dfma_chains<<<blocks, threads, 0, h.stream>>>(iters, 0.999999999, 1e-9, -1.0, out);
    cudaEventRecord(e1, h.stream);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  if (e != cudaSuccess) {
    h.err = std::string("measure_fp64_rate: ") + cudaGetErrorString(e);
    return ICS_ERR_CUDA;
  }
  h.launches += 2;
  *gflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e9;
  return ICS_OK;
}
