// ih_noalloc.cu -- ih_mean_dev_noalloc: the FP64 mean of a device array
// without any allocation.
//
// Who needs it: callers that cannot allocate device memory at the point they
// need a reduction -- a host application that hands the whole GPU memory to a
// fixed arena or pool up front, a real-time loop that must not pay
// cudaMalloc's latency or risk its failure mid-run, or code that has no
// ih_context (creating one allocates the grid's buffers).  ih_mean_dev needs
// a context for its partial-sum scratch; this variant keeps its scratch in a
// fixed device array that is part of the library image instead.
//
// The scratch: g_mean_scratch below, kNoallocBlocks doubles (32 KiB).  Every
// GPU that loads the library holds it until the process exits.  Each call
// writes one partial sum per block into slots [0, blocks) before the second
// kernel reads exactly those slots, so nothing has to be cleared between
// calls; the array keeps the last call's partial sums.  All calls share the
// array: two calls whose kernels overlap on the GPU (different streams, or
// different host threads, on the same device) race on it and must be
// serialised by the caller.
//
// Size limit: n <= kNoallocBlocks * kNoallocChunk = 2^28 doubles (each block
// reduces a fixed chunk of 65536 elements).  Larger n is rejected with
// IH_ERR_TOO_LARGE before anything is launched.
//
// Host code must not pass g_mean_scratch itself to a kernel: in host code the
// name denotes a host-side stand-in, not the device address.  Every call looks
// the device address up with cudaGetSymbolAddress in the context current on
// the calling thread, so a call after cudaDeviceReset (which reloads the
// module at a possibly different address) or under another context of the
// same device gets that context's copy.  The first call in a context may load
// the module there, so make it before any stream capture.
//
// Errors: a failed lookup or launch returns IH_ERR_CUDA and leaves the CUDA
// error pending (cudaPeekAtLastError, not cudaGetLastError), so the caller
// reads its text with cudaGetLastError; an error already pending from the
// caller's own earlier work is reported the same way and is not cleared.
#include <cuda_runtime.h>
#include "../../include/instaheat_gpu.h"

namespace {

constexpr int kNoallocBlocks = 4096;
constexpr long long kNoallocChunk = 65536;
constexpr int kThreads = 256;

static __device__ __align__(256) double g_mean_scratch[kNoallocBlocks];

__device__ double block_sum_na(double v) {
  __shared__ double sh[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kThreads / 32; ++i) r += sh[i];
  return r;
}

// stage 1: block b sums elements [b*chunk, min(n, (b+1)*chunk)) into scratch[b]
__global__ void k_mean_partials_na(const double *__restrict__ f, long long n, double *scratch) {
  const long long lo = (long long)blockIdx.x * kNoallocChunk;
  const long long hi = lo + kNoallocChunk < n ? lo + kNoallocChunk : n;
  double s = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += kThreads) s += f[i];
  s = block_sum_na(s);
  if (threadIdx.x == 0) scratch[blockIdx.x] = s;
}

// stage 2: one block sums the `blocks` partials and writes the mean
__global__ void k_mean_finish_na(const double *scratch, int blocks, long long n, double *out) {
  double s = 0.0;
  for (int b = threadIdx.x; b < blocks; b += kThreads) s += scratch[b];
  s = block_sum_na(s);
  if (threadIdx.x == 0) *out = s / (double)n;
}

// device address of the scratch array in the current context (looked up on
// every call: a plain table lookup once the module is loaded there)
int scratch_for_current_context(double **out) {
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_mean_scratch) != cudaSuccess || !p) return IH_ERR_CUDA;
  *out = static_cast<double *>(p);
  return IH_OK;
}

}  // namespace

extern "C" {

size_t ih_mean_dev_noalloc_max_n(void) { return (size_t)kNoallocBlocks * kNoallocChunk; }

int ih_mean_dev_noalloc(const double *f_dev, size_t n, double *out_dev, void *stream) {
  if (!f_dev || !out_dev || n == 0) return IH_ERR_ARG;
  if (n > ih_mean_dev_noalloc_max_n()) return IH_ERR_TOO_LARGE;
  double *scratch = nullptr;
  int st = scratch_for_current_context(&scratch);
  if (st != IH_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int blocks = (int)((n + kNoallocChunk - 1) / kNoallocChunk);
  k_mean_partials_na<<<blocks, kThreads, 0, s>>>(f_dev, (long long)n, scratch);
  if (cudaPeekAtLastError() != cudaSuccess) return IH_ERR_CUDA;
  k_mean_finish_na<<<1, kThreads, 0, s>>>(scratch, blocks, (long long)n, out_dev);
  if (cudaPeekAtLastError() != cudaSuccess) return IH_ERR_CUDA;
  return IH_OK;
}

}  // extern "C"
