// Linear residual r = b - A x with per-equation L1 sums, allocating nothing.
//
// This is the allocation-free variant of the GMRES residual step (the
// unpreconditioned residual and its L1 sums that gmres::solveDelta computes
// after each restart cycle).  It exists for callers that must not call
// cudaMalloc/cudaFree once they are running: real-time or embedded drivers
// that forbid device allocation after start-up (an allocation can block on
// the driver or fail under memory pressure in the middle of a time step), and
// hosts that own all device memory through their own pool (for example a CFD
// code that hands us its buffers and accounts for every byte on the device).
// Such a caller passes device buffers for the input x, the output r and the
// five L1 sums; the only scratch this kernel needs (per-block partial sums
// and a completion counter) lives in the file-scope device array below,
// which every GPU that loads this library holds until the process exits.
//
// Limits and caveats:
//   * one 256-thread block per 256 cells and 5 partial sums per block, so
//     the array caps the case at NOALLOC_MAX_CELLS = 2,097,152 cells (320 KiB
//     of partials); larger handles are rejected with ICS_ERR_ARG, and so are
//     Harmonic Balance and cyclic handles (A here has neither coupling).
//   * every call shares the array: calls that overlap on the GPU (two
//     streams, two host threads) race on it.  Calls on one stream are safe;
//     each call clears the counter before it launches.
//   * the call runs on the handle's stream and on the handle's device (made
//     current for the call, then restored) and synchronises that stream
//     before it returns, so r and l1 are complete on return.  x must be
//     complete before the call: a caller that wrote it on another stream
//     synchronises that stream (or the device) first.
//   * the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress, with that device current.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "blocks.cuh"
#include "ics_internal.cuh"

// identical to the definition in ics_api.cu (one handle type for the ABI)
struct ics_handle_s {
  ics::Handle h;
};

namespace ics {

constexpr int NOALLOC_THREADS = 256;
constexpr int NOALLOC_MAX_BLOCKS = 8192;
constexpr long NOALLOC_MAX_CELLS = (long)NOALLOC_MAX_BLOCKS * NOALLOC_THREADS;
constexpr int NOALLOC_HEADER = 32;  // 256 bytes: completion counter, then padding
constexpr int NOALLOC_DOUBLES = NOALLOC_HEADER + NOALLOC_MAX_BLOCKS * 5;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_DOUBLES];

// One thread per row: t = A x with FP64 vectors (FP32 or FP64 blocks),
// r = b - t, and the five L1 sums reduced through `scratch`.
template <typename TB>
__global__ void __launch_bounds__(NOALLOC_THREADS)
    k_resid_noalloc(DevMesh m, const TB* __restrict__ blk, const TB* __restrict__ dg, const double* __restrict__ b,
                    const double* __restrict__ x, double* __restrict__ r, double* __restrict__ scratch,
                    double* __restrict__ l1) {
  unsigned int* counter = reinterpret_cast<unsigned int*>(scratch);
  double* partials = scratch + NOALLOC_HEADER;
  double acc[5] = {0, 0, 0, 0, 0};
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < m.N) {
    const int s = c >> 5, lane = c & 31;
    double y[5];
    const TB* D = dg + (size_t)s * 25 * 32 + lane;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      double a = 0.0;
#pragma unroll
      for (int j = 0; j < 5; ++j) a += double(D[(5 * i + j) * 32]) * x[5 * c + j];
      y[i] = a;
    }
    const int base = m.slot_base[s];
    const int ns = m.nslot[c];
    for (int t = 0; t < ns; ++t) {
      const int col = m.scol[(base + t) * 32 + lane];
      double xj[5], yo[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) xj[k] = x[5 * col + k];
      SlotBlock<TB> Bk;
      Bk.load(blk, base + t, lane);
      Bk.mv(m.gamma, xj, yo);
      if (m.vjslot) vj_sub<TB>(m, base + t, lane, col, xj, yo);
#pragma unroll
      for (int i = 0; i < 5; ++i) y[i] += yo[i];
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const double v = b[5 * c + k] - y[k];
      r[5 * c + k] = v;
      acc[k] = fabs(v);
    }
  }
  // block sums -> partials; the last block folds them in block order
  __shared__ double sm[NOALLOC_THREADS / 32][5];
  __shared__ bool amLast;
  const int ln = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    double v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (ln == 0) sm[wp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 5; ++k) {
      double v = 0;
      for (int q = 0; q < NOALLOC_THREADS / 32; ++q) v += sm[q][k];
      partials[blockIdx.x * 5 + k] = v;
    }
    __threadfence();
    amLast = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (amLast && threadIdx.x < 5) {
    __threadfence();
    const volatile double* vp = partials;
    double v = 0;
    for (int q = 0; q < (int)gridDim.x; ++q) v += vp[q * 5 + threadIdx.x];
    l1[threadIdx.x] = v;
  }
}

static std::mutex g_noalloc_mu;
static double* g_noalloc_addr[256] = {};

}  // namespace ics

using namespace ics;

extern "C" int ics_linear_residual_noalloc(ics_handle hh, const double* x, double* r, double* l1) {
  if (!hh || !x || !r || !l1) return ICS_ERR_ARG;
  Handle& h = hh->h;
  if (!h.haveMatrix || !h.haveFlux) {
    h.err = "linear_residual_noalloc needs an assembled Jacobian and a residual";
    return ICS_ERR_STATE;
  }
  if (h.m.nInst > 1) {
    h.err = "linear_residual_noalloc: Harmonic Balance coupling is not provided";
    return ICS_ERR_ARG;
  }
  if (h.m.ncyc > 0) {
    h.err = "linear_residual_noalloc: cyclic couplings are not provided";
    return ICS_ERR_ARG;
  }
  if ((long)h.m.N > NOALLOC_MAX_CELLS) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "linear_residual_noalloc: %d cells exceed the fixed scratch capacity of %ld cells",
                  h.m.N, NOALLOC_MAX_CELLS);
    h.err = buf;
    return ICS_ERR_ARG;
  }
  const int dev = h.device;
  if (dev < 0 || dev >= 256) {
    h.err = "linear_residual_noalloc: device index out of range";
    return ICS_ERR_CUDA;
  }
  // the handle's stream and buffers belong to h.device: make it current for the call
  int prevDev = -1;
  cudaError_t e = cudaGetDevice(&prevDev);
  if (e == cudaSuccess && prevDev != dev) e = cudaSetDevice(dev);
  if (e != cudaSuccess) {
    h.err = std::string("linear_residual_noalloc: ") + cudaGetErrorString(e);
    return ICS_ERR_CUDA;
  }
  struct Restore {
    int prev, dev;
    ~Restore() {
      if (prev >= 0 && prev != dev) cudaSetDevice(prev);
    }
  } restore{prevDev, dev};
  double* scratch = nullptr;
  {
    // set-up once per device, with that device current
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        h.err = std::string("linear_residual_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
        return ICS_ERR_CUDA;
      }
      g_noalloc_addr[dev] = static_cast<double*>(p);
    }
    scratch = g_noalloc_addr[dev];
  }
  // the array keeps the previous call's contents: the counter must start at zero
  e = cudaMemsetAsync(scratch, 0, sizeof(unsigned int), h.stream);
  if (e != cudaSuccess) {
    h.err = std::string("linear_residual_noalloc: ") + cudaGetErrorString(e);
    return ICS_ERR_CUDA;
  }
  const int blocks = (h.m.N + NOALLOC_THREADS - 1) / NOALLOC_THREADS;
  if (h.jacPrecision == ICS_PREC_MIXED)
    k_resid_noalloc<float><<<blocks, NOALLOC_THREADS, 0, h.stream>>>(h.m, (const float*)h.blk, (const float*)h.dg,
                                                                     h.src, x, r, scratch, l1);
  else
    k_resid_noalloc<double><<<blocks, NOALLOC_THREADS, 0, h.stream>>>(h.m, (const double*)h.blk, (const double*)h.dg,
                                                                      h.src, x, r, scratch, l1);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
  if (e != cudaSuccess) {
    h.err = std::string("linear_residual_noalloc: ") + cudaGetErrorString(e);
    return ICS_ERR_CUDA;
  }
  return ICS_OK;
}
