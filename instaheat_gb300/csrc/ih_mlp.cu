// ih_mlp.cu -- the learned step-size proposer: a 12 -> 64 -> 64 -> 1 MLP with
// GELU activations, BF16 weights and FP32 accumulation, trained and run by
// hand-written kernels.  No reference counterpart (the reference's step
// sizes come from its controller alone, dopri853.c:505-540); here the
// DOPRI853 error estimate still accepts or rejects every step and the
// controller remains the fallback.
//
// Parameters (flat FP32 master copy, IH_MLP_NPARAMS floats):
//   W1[12][64], b1[64], W2[64][64], b2[64], W3[64], b3
// The forward and backward passes read a BF16 copy of the weights (refreshed
// after every optimiser step) and accumulate in FP32; Adam updates the FP32
// master copy.  Inputs are normalised with the stored per-feature mean/std;
// the output is de-normalised to log(dt).
//
// Training runs as one kernel launch on one CTA: the dataset (at most a few
// thousand step-log rows) sits in global memory, every iteration draws a
// minibatch with a counter-based generator, does forward + backward for one
// sample per thread, reduces the weight gradients in shared memory and
// applies Adam.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>
#include <string>
#include <vector>
#include "../../include/instaheat_gpu.h"

namespace {

constexpr int NI = IH_MLP_INPUTS, NH = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NI * NH, OFF_W2 = OFF_B1 + NH;
constexpr int OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH;
constexpr int NP = OFF_B3 + 1;
static_assert(NP == IH_MLP_NPARAMS, "parameter count");
constexpr int BT = 128;  // samples per minibatch (one per thread)

__device__ __forceinline__ float gelu(float x) {
  // tanh form of GELU
  const float c = 0.7978845608028654f;  // sqrt(2/pi)
  return 0.5f * x * (1.f + tanhf(c * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float c = 0.7978845608028654f;
  const float u = c * (x + 0.044715f * x * x * x);
  const float t = tanhf(u);
  const float du = c * (1.f + 3.f * 0.044715f * x * x);
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * du;
}

struct Norm {
  float mean[NI], std[NI];
  float out_mean, out_std;
};

// weights BF16 -> FP32 in shared memory
__device__ void stage_weights(const __nv_bfloat16 *wb, float *sw) {
  for (int i = threadIdx.x; i < NP; i += blockDim.x) sw[i] = __bfloat162float(wb[i]);
}

// forward of one (normalised) sample; keeps z1, z2, h1, h2 for backward
__device__ float forward_one(const float *sw, const float *x, float *z1, float *h1, float *z2,
                             float *h2) {
  for (int j = 0; j < NH; ++j) {
    float a = sw[OFF_B1 + j];
    for (int i = 0; i < NI; ++i) a = fmaf(x[i], sw[OFF_W1 + i * NH + j], a);
    z1[j] = a;
    h1[j] = gelu(a);
  }
  for (int j = 0; j < NH; ++j) {
    float a = sw[OFF_B2 + j];
    for (int i = 0; i < NH; ++i) a = fmaf(h1[i], sw[OFF_W2 + i * NH + j], a);
    z2[j] = a;
    h2[j] = gelu(a);
  }
  float o = sw[OFF_B3];
  for (int i = 0; i < NH; ++i) o = fmaf(h2[i], sw[OFF_W3 + i], o);
  return o;
}

__device__ __forceinline__ void normalise(const float *xin, const Norm &nm, float *x) {
  for (int i = 0; i < NI; ++i) x[i] = (xin[i] - nm.mean[i]) / nm.std[i];
}

// inference: one thread per row, output log(dt)
__global__ void k_mlp_forward(const __nv_bfloat16 *wb, Norm nm, const float *X, int n, float *Y) {
  extern __shared__ float sw[];
  stage_weights(wb, sw);
  __syncthreads();
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    float x[NI], z1[NH], h1[NH], z2[NH], h2[NH];
    normalise(X + (size_t)r * NI, nm, x);
    const float o = forward_one(sw, x, z1, h1, z2, h2);
    Y[r] = o * nm.out_std + nm.out_mean;
  }
}

__device__ __forceinline__ unsigned hash32(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// Gradient of the mean squared error (in normalised output units) over rows
// idx[0..bt) of the data set, accumulated into g (NP floats in shared memory).
// Thread t < bt handles row idx[t]; per-sample activations go through shared
// memory so that the weight gradients are reduced without atomics.
__device__ float batch_gradients(const float *sw, const Norm &nm, const float *X, const float *Y,
                                 const int *idx, int bt, float *g, float *s_x, float *s_h1,
                                 float *s_dz1, float *s_dz2, float *s_h2, float *s_dy,
                                 float *s_loss) {
  const int t = threadIdx.x;
  for (int i = t; i < NP; i += blockDim.x) g[i] = 0.f;
  if (t < bt) {
    float x[NI], z1[NH], h1[NH], z2[NH], h2[NH];
    const int r = idx[t];
    normalise(X + (size_t)r * NI, nm, x);
    const float o = forward_one(sw, x, z1, h1, z2, h2);
    const float target = (Y[r] - nm.out_mean) / nm.out_std;
    const float diff = o - target;
    s_loss[t] = diff * diff;
    const float dy = 2.f * diff / (float)bt;
    s_dy[t] = dy;
    float dz2[NH];
    for (int j = 0; j < NH; ++j) dz2[j] = dy * sw[OFF_W3 + j] * gelu_grad(z2[j]);
    for (int i = 0; i < NH; ++i) {
      float a = 0.f;
      for (int j = 0; j < NH; ++j) a = fmaf(sw[OFF_W2 + i * NH + j], dz2[j], a);
      s_dz1[t * NH + i] = a * gelu_grad(z1[i]);
    }
    for (int i = 0; i < NI; ++i) s_x[t * NI + i] = x[i];
    for (int j = 0; j < NH; ++j) {
      s_h1[t * NH + j] = h1[j];
      s_h2[t * NH + j] = h2[j];
      s_dz2[t * NH + j] = dz2[j];
    }
  } else if (t < BT) {
    s_loss[t] = 0.f;
  }
  __syncthreads();
  // weight gradients: each thread owns a strided set of parameters
  for (int p = t; p < NP; p += blockDim.x) {
    float a = 0.f;
    if (p < OFF_B1) {
      const int i = p / NH, j = p % NH;
      for (int b = 0; b < bt; ++b) a = fmaf(s_x[b * NI + i], s_dz1[b * NH + j], a);
    } else if (p < OFF_W2) {
      const int j = p - OFF_B1;
      for (int b = 0; b < bt; ++b) a += s_dz1[b * NH + j];
    } else if (p < OFF_B2) {
      const int q = p - OFF_W2, i = q / NH, j = q % NH;
      for (int b = 0; b < bt; ++b) a = fmaf(s_h1[b * NH + i], s_dz2[b * NH + j], a);
    } else if (p < OFF_W3) {
      const int j = p - OFF_B2;
      for (int b = 0; b < bt; ++b) a += s_dz2[b * NH + j];
    } else if (p < OFF_B3) {
      const int i = p - OFF_W3;
      for (int b = 0; b < bt; ++b) a = fmaf(s_h2[b * NH + i], s_dy[b], a);
    } else {
      for (int b = 0; b < bt; ++b) a += s_dy[b];
    }
    g[p] = a;
  }
  __syncthreads();
  float l = 0.f;
  if (t == 0)
    for (int b = 0; b < bt; ++b) l += s_loss[b];
  return l / (float)(bt > 0 ? bt : 1);
}

// shared-memory layout of the training / gradient kernels (floats)
constexpr int SM_W = NP, SM_G = NP, SM_X = BT * NI, SM_H = BT * NH;
constexpr size_t kTrainSmem =
    sizeof(float) * (SM_W + SM_G + SM_X + 4 * SM_H + 2 * BT) + sizeof(int) * BT;

// full-batch gradient (summed over chunks of BT rows) into gout, loss into lout
__global__ void k_mlp_gradients(const __nv_bfloat16 *wb, Norm nm, const float *X, const float *Y,
                                int n, float *gout, float *lout) {
  extern __shared__ float sm[];
  float *sw = sm, *g = sw + SM_W, *s_x = g + SM_G, *s_h1 = s_x + SM_X, *s_dz1 = s_h1 + SM_H;
  float *s_dz2 = s_dz1 + SM_H, *s_h2 = s_dz2 + SM_H, *s_dy = s_h2 + SM_H, *s_loss = s_dy + BT;
  int *idx = reinterpret_cast<int *>(s_loss + BT);
  stage_weights(wb, sw);
  for (int p = threadIdx.x; p < NP; p += blockDim.x) gout[p] = 0.f;
  __syncthreads();
  float ltot = 0.f;
  for (int c0 = 0; c0 < n; c0 += BT) {
    const int bt = min(BT, n - c0);
    if (threadIdx.x < BT) idx[threadIdx.x] = c0 + threadIdx.x;
    __syncthreads();
    // per-chunk gradients are of the chunk mean; weight them by bt / n
    const float l = batch_gradients(sw, nm, X, Y, idx, bt, g, s_x, s_h1, s_dz1, s_dz2, s_h2,
                                    s_dy, s_loss);
    for (int p = threadIdx.x; p < NP; p += blockDim.x) gout[p] += g[p] * (float)bt / (float)n;
    if (threadIdx.x == 0) ltot += l * (float)bt / (float)n;
    __syncthreads();
  }
  if (threadIdx.x == 0) *lout = ltot;
}

// Adam training, everything in one launch on one CTA
__global__ void k_mlp_train(float *w, float *m, float *v, __nv_bfloat16 *wb, Norm nm,
                            const float *X, const float *Y, int n, int iters, int bt, float lr,
                            unsigned seed, float *loss_hist) {
  extern __shared__ float sm[];
  float *sw = sm, *g = sw + SM_W, *s_x = g + SM_G, *s_h1 = s_x + SM_X, *s_dz1 = s_h1 + SM_H;
  float *s_dz2 = s_dz1 + SM_H, *s_h2 = s_dz2 + SM_H, *s_dy = s_h2 + SM_H, *s_loss = s_dy + BT;
  int *idx = reinterpret_cast<int *>(s_loss + BT);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int it = 0; it < iters; ++it) {
    for (int p = threadIdx.x; p < NP; p += blockDim.x) sw[p] = __bfloat162float(wb[p]);
    if (threadIdx.x < bt) idx[threadIdx.x] = (int)(hash32(seed * 2654435761U + it * 1315423911U +
                                                         threadIdx.x) % (unsigned)n);
    __syncthreads();
    const float l = batch_gradients(sw, nm, X, Y, idx, bt, g, s_x, s_h1, s_dz1, s_dz2, s_h2,
                                    s_dy, s_loss);
    if (threadIdx.x == 0) loss_hist[it] = l;
    const float c1 = 1.f - powf(b1, (float)(it + 1)), c2 = 1.f - powf(b2, (float)(it + 1));
    for (int p = threadIdx.x; p < NP; p += blockDim.x) {
      const float gp = g[p];
      const float mp = b1 * m[p] + (1.f - b1) * gp;
      const float vp = b2 * v[p] + (1.f - b2) * gp * gp;
      m[p] = mp;
      v[p] = vp;
      const float wp = w[p] - lr * (mp / c1) / (sqrtf(vp / c2) + eps);
      w[p] = wp;
      wb[p] = __float2bfloat16(wp);
    }
    __syncthreads();
  }
}

__global__ void k_refresh_bf16(const float *w, __nv_bfloat16 *wb) {
  for (int p = threadIdx.x; p < NP; p += blockDim.x) wb[p] = __float2bfloat16(w[p]);
}

}  // namespace

struct ih_mlp {
  float *w = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16 *wb = nullptr;
  Norm nm{};
  int device = 0;
  std::string err;
};

static int mlp_cuda(ih_mlp *h, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return IH_OK;
  h->err = std::string(what) + ": " + cudaGetErrorString(e);
  return IH_ERR_CUDA;
}
#define MLP_CK(h, call)                              \
  do {                                               \
    int s_ = mlp_cuda((h), (call), #call);           \
    if (s_ != IH_OK) return s_;                      \
  } while (0)

extern "C" {

int ih_mlp_create(int device, unsigned seed, ih_mlp **out) {
  if (!out) return IH_ERR_ARG;
  *out = nullptr;
  ih_mlp *h = new ih_mlp();
  h->device = device;
  for (int i = 0; i < NI; ++i) {
    h->nm.mean[i] = 0.f;
    h->nm.std[i] = 1.f;
  }
  h->nm.out_mean = 0.f;
  h->nm.out_std = 1.f;
  if (cudaSetDevice(device) != cudaSuccess || cudaMalloc(&h->w, sizeof(float) * NP) != cudaSuccess ||
      cudaMalloc(&h->m, sizeof(float) * NP) != cudaSuccess ||
      cudaMalloc(&h->v, sizeof(float) * NP) != cudaSuccess ||
      cudaMalloc(&h->wb, sizeof(__nv_bfloat16) * NP) != cudaSuccess) {
    ih_mlp_destroy(h);
    return IH_ERR_ALLOC;
  }
  // Glorot-uniform initial weights from a host LCG, zero biases
  std::vector<float> w(NP, 0.f);
  unsigned long long s = 0x9E3779B97F4A7C15ULL ^ seed;
  auto uni = [&s]() {
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
  };
  auto fill = [&](int off, int fan_in, int fan_out) {
    const double a = sqrt(6.0 / (fan_in + fan_out));
    for (int i = 0; i < fan_in * fan_out; ++i) w[off + i] = (float)((2.0 * uni() - 1.0) * a);
  };
  fill(OFF_W1, NI, NH);
  fill(OFF_W2, NH, NH);
  fill(OFF_W3, NH, 1);
  int st = ih_mlp_set_params(h, w.data());
  if (st != IH_OK) {
    ih_mlp_destroy(h);
    return st;
  }
  *out = h;
  return IH_OK;
}

void ih_mlp_destroy(ih_mlp *h) {
  if (!h) return;
  if (h->w) cudaFree(h->w);
  if (h->m) cudaFree(h->m);
  if (h->v) cudaFree(h->v);
  if (h->wb) cudaFree(h->wb);
  delete h;
}

const char *ih_mlp_last_error(const ih_mlp *h) { return h ? h->err.c_str() : "null"; }

int ih_mlp_set_params(ih_mlp *h, const float *p) {
  if (!h || !p) return IH_ERR_ARG;
  MLP_CK(h, cudaSetDevice(h->device));
  MLP_CK(h, cudaMemcpy(h->w, p, sizeof(float) * NP, cudaMemcpyHostToDevice));
  MLP_CK(h, cudaMemset(h->m, 0, sizeof(float) * NP));
  MLP_CK(h, cudaMemset(h->v, 0, sizeof(float) * NP));
  k_refresh_bf16<<<1, 256>>>(h->w, h->wb);
  MLP_CK(h, cudaGetLastError());
  MLP_CK(h, cudaDeviceSynchronize());
  return IH_OK;
}

int ih_mlp_get_params(ih_mlp *h, float *p) {
  if (!h || !p) return IH_ERR_ARG;
  MLP_CK(h, cudaSetDevice(h->device));
  MLP_CK(h, cudaMemcpy(p, h->w, sizeof(float) * NP, cudaMemcpyDeviceToHost));
  return IH_OK;
}

int ih_mlp_set_norm(ih_mlp *h, const float *in_mean, const float *in_std, float out_mean,
                    float out_std) {
  if (!h || !in_mean || !in_std || !(out_std > 0.f)) return IH_ERR_ARG;
  for (int i = 0; i < NI; ++i) {
    if (!(in_std[i] > 0.f)) return IH_ERR_ARG;
    h->nm.mean[i] = in_mean[i];
    h->nm.std[i] = in_std[i];
  }
  h->nm.out_mean = out_mean;
  h->nm.out_std = out_std;
  return IH_OK;
}

int ih_mlp_forward(ih_mlp *h, const float *x, int n, float *y) {
  if (!h || !x || !y || n < 1) return IH_ERR_ARG;
  MLP_CK(h, cudaSetDevice(h->device));
  float *dx = nullptr, *dy = nullptr;
  MLP_CK(h, cudaMalloc(&dx, sizeof(float) * NI * (size_t)n));
  if (cudaMalloc(&dy, sizeof(float) * (size_t)n) != cudaSuccess) {
    cudaFree(dx);
    return IH_ERR_ALLOC;
  }
  int st = IH_OK;
  if (cudaMemcpy(dx, x, sizeof(float) * NI * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess)
    st = IH_ERR_CUDA;
  if (st == IH_OK) {
    const int blocks = (n + 127) / 128;
    k_mlp_forward<<<blocks, 128, sizeof(float) * NP>>>(h->wb, h->nm, dx, n, dy);
    if (cudaGetLastError() != cudaSuccess) st = IH_ERR_CUDA;
  }
  if (st == IH_OK && cudaMemcpy(y, dy, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
    st = IH_ERR_CUDA;
  cudaFree(dx);
  cudaFree(dy);
  return st;
}

int ih_mlp_gradients(ih_mlp *h, const float *x, const float *y, int n, float *grad, float *loss) {
  if (!h || !x || !y || !grad || n < 1) return IH_ERR_ARG;
  MLP_CK(h, cudaSetDevice(h->device));
  float *dx = nullptr, *dy = nullptr, *dg = nullptr;
  size_t need = sizeof(float) * ((size_t)NI * n + n + NP + 1);
  float *blk = nullptr;
  MLP_CK(h, cudaMalloc(&blk, need));
  dx = blk;
  dy = dx + (size_t)NI * n;
  dg = dy + n;
  int st = IH_OK;
  if (cudaMemcpy(dx, x, sizeof(float) * NI * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess)
    st = IH_ERR_CUDA;
  if (st == IH_OK) {
    cudaFuncSetAttribute(k_mlp_gradients, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kTrainSmem);
    k_mlp_gradients<<<1, 256, kTrainSmem>>>(h->wb, h->nm, dx, dy, n, dg, dg + NP);
    if (cudaGetLastError() != cudaSuccess) st = IH_ERR_CUDA;
  }
  float l = 0.f;
  if (st == IH_OK && (cudaMemcpy(grad, dg, sizeof(float) * NP, cudaMemcpyDeviceToHost) != cudaSuccess ||
                      cudaMemcpy(&l, dg + NP, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess))
    st = IH_ERR_CUDA;
  if (loss) *loss = l;
  cudaFree(blk);
  return st;
}

int ih_mlp_train(ih_mlp *h, const float *x, const float *y, int n, int iters, int batch, float lr,
                 unsigned seed, float *loss_hist) {
  if (!h || !x || !y || n < 1 || iters < 1 || batch < 1 || batch > BT || !(lr > 0.f))
    return IH_ERR_ARG;
  MLP_CK(h, cudaSetDevice(h->device));
  float *blk = nullptr;
  size_t need = sizeof(float) * ((size_t)NI * n + n + iters);
  MLP_CK(h, cudaMalloc(&blk, need));
  float *dx = blk, *dy = dx + (size_t)NI * n, *dl = dy + n;
  int st = IH_OK;
  if (cudaMemcpy(dx, x, sizeof(float) * NI * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess)
    st = IH_ERR_CUDA;
  if (st == IH_OK) {
    cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem);
    k_mlp_train<<<1, 256, kTrainSmem>>>(h->w, h->m, h->v, h->wb, h->nm, dx, dy, n, iters, batch, lr,
                                        seed, dl);
    if (cudaGetLastError() != cudaSuccess) st = IH_ERR_CUDA;
  }
  if (st == IH_OK && cudaDeviceSynchronize() != cudaSuccess) st = IH_ERR_CUDA;
  if (st == IH_OK && loss_hist &&
      cudaMemcpy(loss_hist, dl, sizeof(float) * iters, cudaMemcpyDeviceToHost) != cudaSuccess)
    st = IH_ERR_CUDA;
  cudaFree(blk);
  return st;
}

}  // extern "C"

namespace ih {
// Inference on device buffers on a given stream (used by the stepper).
int mlp_forward_async(ih_mlp *h, const float *dx, int n, float *dy, cudaStream_t s) {
  if (!h) return IH_ERR_ARG;
  k_mlp_forward<<<(n + 127) / 128, 128, sizeof(float) * NP, s>>>(h->wb, h->nm, dx, n, dy);
  return cudaGetLastError() == cudaSuccess ? IH_OK : IH_ERR_CUDA;
}
}  // namespace ih

extern "C" {

// BF16 weights as the forward pass sees them (for checks), NP floats
int ih_mlp_get_bf16_params(ih_mlp *h, float *p) {
  if (!h || !p) return IH_ERR_ARG;
  std::vector<__nv_bfloat16> b(NP);
  MLP_CK(h, cudaSetDevice(h->device));
  MLP_CK(h, cudaMemcpy(b.data(), h->wb, sizeof(__nv_bfloat16) * NP, cudaMemcpyDeviceToHost));
  for (int i = 0; i < NP; ++i) p[i] = __bfloat162float(b[i]);
  return IH_OK;
}

}  // extern "C"
