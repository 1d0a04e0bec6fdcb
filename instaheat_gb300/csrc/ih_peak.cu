// ih_peak.cu -- measured FP64 FMA throughput of the current GPU, the
// denominator of the plain FP64 form's ALU roofline.  No reference
// counterpart (the reference runs on CPUs).
//
// Each thread runs kChains independent chains x <- x * m + c (one DFMA per
// link) for `iters` links, so every warp keeps kChains DFMAs in flight; the
// grid is 8 CTAs of 256 threads per SM.  Throughput = 2 flops per DFMA over
// the CUDA-event time of the launch (best of `reps` launches after one
// warm-up).  The chains' sum is written only if it equals an impossible
// value, which keeps the arithmetic alive without a store per thread.
#include <cuda_runtime.h>
#include "../../include/instaheat_gpu.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void k_fp64_fma_chains(double *sink, int iters, double m, double c) {
  double x[kChains];
#pragma unroll
  for (int j = 0; j < kChains; ++j) x[j] = 1.0 + 1e-3 * (threadIdx.x + j);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < kChains; ++j) x[j] = fma(x[j], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < kChains; ++j) s += x[j];
  if (s == -1.0) sink[0] = s;
}

}  // namespace

extern "C" int ih_fp64_fma_peak(int device, int iters, int reps, double *tflops) {
  if (!tflops || iters < 1 || reps < 1) return IH_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return IH_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return IH_ERR_CUDA;
  double *sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = IH_ERR_CUDA;
  const int blocks = sms * 8;
  float best = 0.f;
  if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) return IH_ERR_CUDA;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) goto done;
  k_fp64_fma_chains<<<blocks, kThreads>>>(sink, iters, 0.999999999, 1e-9);
  if (cudaDeviceSynchronize() != cudaSuccess) goto done;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0);
    k_fp64_fma_chains<<<blocks, kThreads>>>(sink, iters, 0.999999999, 1e-9);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) goto done;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r == 0 || ms < best) best = ms;
  }
  *tflops = 2.0 * kChains * (double)iters * blocks * kThreads / (best * 1e-3) / 1e12;
  st = IH_OK;
done:
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(sink);
  return st;
}
