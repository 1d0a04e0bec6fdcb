// ih_fft.cu -- 3D real FFTs for power-of-two grids on GB300, FP32 and FP64.
//
// Replaces the reference's FFTW calls (src/toolbox.c:806-827; plans
// src/setup.c:524-554) with FFTW's conventions: r2c is the unnormalised
// exp(-2 pi i jk/n) transform into the half spectrum [nx][ny][nz/2+1], c2r the
// unnormalised exp(+2 pi i jk/n) inverse.
//
// Structure: three passes per transform (z, y, x), each one kernel.  Every
// pencil of length L = R1*R2 is transformed in two register steps with one
// shared-memory exchange:
//   step 1: thread (pencil, n1) holds x[n1 + R1*n2], n2 < R2, does an
//           in-register R2-point DFT and multiplies by exp(-+2 pi i n1 k2/L);
//   step 2: thread (pencil, k2) gathers the R1 values of its k2, does an
//           in-register R1-point DFT and owns X[k2 + R2*k1].
// The in-register DFTs are radix-2 decimation-in-frequency networks whose
// loop structure and bit reversal are resolved at compile time; their
// twiddles come from a table exp(-2 pi i m/L) computed once in FP64 on the
// host and staged in shared memory.  x and y passes load straight from global
// memory into registers (tiles of B pencils, B = one 128-byte line of complex
// values: 16 FP32 / 8 FP64) and store straight back.  z passes work on whole
// contiguous rows (a real row of nz values packed as nz/2 complex, with the
// even/odd split) and stage the rows in shared memory for the split.
//
// Fused passes (the RHS never materialises ik*phihat or the six real
// products d_i phi d_j phi):
//   fft_x_deriv4_inv -- reads phihat once, multiplies by i k_x, i k_y, i k_z,
//                       -k^2 (all / N) and runs four inverse x transforms;
//   fft_z_rhs_fused  -- four inverse z transforms, the pointwise energy
//                       density / pressure / gradient terms with FP64 block
//                       sums, and six forward z transforms of the GW source
//                       products, all on one tile of rows.
#include <math.h>
#include <mutex>
#include <utility>
#include <unordered_map>
#include "ih_internal.cuh"
#include "ih_tensor.cuh"
#include "ih_fftcore.cuh"

namespace ih {

template <typename T> __host__ __device__ constexpr int tileB() { return 128 / (int)(2 * sizeof(T)); }

// L = R1 * R2: threads per pencil in step 1, points per thread in step 1
template <int L> struct Fac;
template <> struct Fac<4> { static constexpr int R1 = 2, R2 = 2; };
template <> struct Fac<8> { static constexpr int R1 = 4, R2 = 2; };
template <> struct Fac<16> { static constexpr int R1 = 4, R2 = 4; };
template <> struct Fac<32> { static constexpr int R1 = 8, R2 = 4; };
template <> struct Fac<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct Fac<128> { static constexpr int R1 = 16, R2 = 8; };
template <> struct Fac<256> { static constexpr int R1 = 16, R2 = 16; };
template <> struct Fac<512> { static constexpr int R1 = 16, R2 = 32; };

template <int L> __host__ __device__ constexpr int max_r() {
  return Fac<L>::R1 > Fac<L>::R2 ? Fac<L>::R1 : Fac<L>::R2;
}
__host__ __device__ constexpr int round_warp(int n) { return n < 32 ? 32 : (n + 31) / 32 * 32; }
// threads of a pass over B pencils (rows) of length L: one per pencil and
// register column of the wider step
template <int L, int B> __host__ __device__ constexpr int pass_threads() {
  return round_warp(max_r<L>() * B);
}
// Row of the exchange buffer [L][B] of the two-step kernels (no padding).
// A warp's access touches one row per thread group q (rows q R2 + k2 when
// step 1 writes, q R1 + n1 when step 2 writes, consecutive rows when the
// next step reads).  With half-line rows (64 bytes) rows of equal parity
// share a half of the banks, and R1, R2 >= 8 make the written rows of one
// warp all even or all odd: the row is swapped with its neighbour (r ^ 1) on
// alternate blocks of R1 (and R2) rows, which puts the groups of every such
// access on both halves, a permutation of the rows.
template <int L> __device__ __forceinline__ int xrow(int r) {
  constexpr int a = clog2(Fac<L>::R1), b = clog2(Fac<L>::R2);
  const int f = (a == b) ? (r >> a) : ((r >> a) ^ (r >> b));
  return r ^ (f & 1);
}
// exp(sign 2 pi i m / L) from the table exp(-2 pi i m/L)
// Butterflies per thread per radix-4 stage (2K per radix-2 stage); the
// launchers size CTAs so that B*L <= 4*K*nt.
constexpr int kFftK = 2;

// In-place Stockham FFT of B pencils of length L (a power of two) held in
// s[L][P] (P >= B).  tw[k] = exp(-2 pi i k/L); sign -1 forward, +1 backward.
// Requires B*L <= 4*K*nt.  Two barriers per stage: every thread gathers its
// butterfly inputs into registers before any thread scatters results.
template <typename T, int B, int K>
__device__ void smem_fft(C2<T> *s, int L, int P, const C2<T> *tw, int sign, int tid, int nt) {
  constexpr int LB = clog2(B);
  int Lc = L, lst = 0;
  while (Lc > 1) {
    const int st = 1 << lst;
    if ((Lc & 3) == 0) {
      const int m = Lc >> 2;
      const int nb = (B * L) >> 2;
      C2<T> v[4 * K];
#pragma unroll
      for (int kk = 0; kk < K; ++kk) {
        const int u = tid + kk * nt;
        if (u < nb) {
          const int b = u & (B - 1), w = u >> LB, q = w & (st - 1), pp = w >> lst;
#pragma unroll
          for (int t = 0; t < 4; ++t) v[kk * 4 + t] = s[(q + ((pp + t * m) << lst)) * P + b];
        }
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < K; ++kk) {
        const int u = tid + kk * nt;
        if (u < nb) {
          const int b = u & (B - 1), w = u >> LB, q = w & (st - 1), pp = w >> lst;
          C2<T> x0 = v[kk * 4], x1 = v[kk * 4 + 1], x2 = v[kk * 4 + 2], x3 = v[kk * 4 + 3];
          C2<T> s02 = cadd(x0, x2), d02 = csub(x0, x2);
          C2<T> s13 = cadd(x1, x3), d13 = csub(x1, x3);
          // (sign*i) * d13
          C2<T> j13 = mk2<T>(-(T)sign * d13.y, (T)sign * d13.x);
          C2<T> y0 = cadd(s02, s13), y2 = csub(s02, s13);
          C2<T> y1 = cadd(d02, j13), y3 = csub(d02, j13);
          const int base = (q + ((4 * pp) << lst)) * P + b;
          const int sp = st * P;
          s[base] = y0;
          if (pp == 0) {
            s[base + sp] = y1;
            s[base + 2 * sp] = y2;
            s[base + 3 * sp] = y3;
          } else {
            const int ti = pp << lst;
            C2<T> w1 = tw[ti], w2 = tw[2 * ti], w3 = tw[3 * ti];
            if (sign > 0) {
              w1.y = -w1.y;
              w2.y = -w2.y;
              w3.y = -w3.y;
            }
            s[base + sp] = cmul(y1, w1);
            s[base + 2 * sp] = cmul(y2, w2);
            s[base + 3 * sp] = cmul(y3, w3);
          }
        }
      }
      Lc = m;
      lst += 2;
    } else {
      const int m = Lc >> 1;
      const int nb = (B * L) >> 1;
      C2<T> v[4 * K];
#pragma unroll
      for (int kk = 0; kk < 2 * K; ++kk) {
        const int u = tid + kk * nt;
        if (u < nb) {
          const int b = u & (B - 1), w = u >> LB, q = w & (st - 1), pp = w >> lst;
          v[kk * 2] = s[(q + (pp << lst)) * P + b];
          v[kk * 2 + 1] = s[(q + ((pp + m) << lst)) * P + b];
        }
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < 2 * K; ++kk) {
        const int u = tid + kk * nt;
        if (u < nb) {
          const int b = u & (B - 1), w = u >> LB, q = w & (st - 1), pp = w >> lst;
          C2<T> a = v[kk * 2], c = v[kk * 2 + 1];
          C2<T> y0 = cadd(a, c), y1 = csub(a, c);
          if (pp != 0) {
            C2<T> w1 = tw[pp << lst];
            if (sign > 0) w1.y = -w1.y;
            y1 = cmul(y1, w1);
          }
          const int base = (q + ((2 * pp) << lst)) * P + b;
          s[base] = y0;
          s[base + st * P] = y1;
        }
      }
      Lc = m;
      lst += 1;
    }
    __syncthreads();
  }
}

// The same Stockham stages for any L = 2^a 3^b: radix 4 while 4 divides
// the remaining length, then 2, then 3; the index arithmetic divides by the
// stride (no longer a power of two after a radix-3 stage).  A radix-3 stage
// is y0 = x0 + s, y1,2 = x0 - s/2 +- sign i (sqrt 3/2) d with s = x1 + x2,
// d = x1 - x2.  Requires B*L <= 4*K*nt like smem_fft.
template <typename T, int B, int K>
__device__ void smem_fft_g(C2<T> *s, int L, int P, const C2<T> *tw, int sign, int tid, int nt) {
  constexpr int LB = clog2(B);
  constexpr int K3 = (4 * K + 2) / 3;  // radix-3 butterflies per thread
  const T h3 = (T)0.86602540378443864676;
  int Lc = L, st = 1;
  while (Lc > 1) {
    const int r = (Lc % 4 == 0) ? 4 : ((Lc % 2 == 0) ? 2 : 3);
    const int m = Lc / r;
    const int nb = (B * L) / r;
    const int bpt = r == 4 ? K : (r == 2 ? 2 * K : K3);
    C2<T> v[4 * K + 2];
    for (int kk = 0; kk < bpt; ++kk) {
      const int u = tid + kk * nt;
      if (u < nb) {
        const int b = u & (B - 1), w = u >> LB, q = w % st, pp = w / st;
        for (int t = 0; t < r; ++t) v[kk * r + t] = s[(q + (pp + t * m) * st) * P + b];
      }
    }
    __syncthreads();
    for (int kk = 0; kk < bpt; ++kk) {
      const int u = tid + kk * nt;
      if (u >= nb) continue;
      const int b = u & (B - 1), w = u >> LB, q = w % st, pp = w / st;
      C2<T> y[4];
      if (r == 4) {
        const C2<T> x0 = v[kk * 4], x1 = v[kk * 4 + 1], x2 = v[kk * 4 + 2], x3 = v[kk * 4 + 3];
        const C2<T> s02 = cadd(x0, x2), d02 = csub(x0, x2);
        const C2<T> s13 = cadd(x1, x3), d13 = csub(x1, x3);
        const C2<T> j13 = mk2<T>(-(T)sign * d13.y, (T)sign * d13.x);  // (sign i) d13
        y[0] = cadd(s02, s13);
        y[2] = csub(s02, s13);
        y[1] = cadd(d02, j13);
        y[3] = csub(d02, j13);
      } else if (r == 2) {
        const C2<T> a = v[kk * 2], c = v[kk * 2 + 1];
        y[0] = cadd(a, c);
        y[1] = csub(a, c);
      } else {
        const C2<T> x0 = v[kk * 3], x1 = v[kk * 3 + 1], x2 = v[kk * 3 + 2];
        const C2<T> s12 = cadd(x1, x2), d12 = csub(x1, x2);
        const C2<T> tq = mk2<T>(x0.x - (T)0.5 * s12.x, x0.y - (T)0.5 * s12.y);
        const C2<T> jd = mk2<T>(-(T)sign * h3 * d12.y, (T)sign * h3 * d12.x);
        y[0] = cadd(x0, s12);
        y[1] = cadd(tq, jd);
        y[2] = csub(tq, jd);
      }
      const int base = (q + r * pp * st) * P + b;
      s[base] = y[0];
      for (int t = 1; t < r; ++t) {
        C2<T> yt = y[t];
        if (pp != 0) {
          C2<T> wt = tw[t * pp * st];
          if (sign > 0) wt.y = -wt.y;
          yt = cmul(yt, wt);
        }
        s[base + t * st * P] = yt;
      }
    }
    Lc = m;
    st *= r;
    __syncthreads();
  }
}

template <typename V>
__device__ __forceinline__ V twid(const V *tw, int m, int sign) {
  V w = tw[m];
  if (sign > 0) w.y = -w.y;
  return w;
}

template <typename V>
__device__ __forceinline__ void load_table(V *dst, const V *src, int n, int tid, int nt) {
  for (int i = tid; i < n; i += nt) dst[i] = src[i];
}

// ---------------------------------------------------------------------------
// Complex passes along x (axis 0) or y (axis 1), in place, batched over
// arrays (blockIdx.z).  A CTA transforms a tile of B pencils: columns
// z0..z0+B-1 of one plane, element j of a pencil at j * sj.  Two engines,
// chosen per axis by the autotuner (fft_autotune):
//   Stockham  -- the tile is staged in shared memory [L][B+1] and transformed
//                in place by radix-4/2 Stockham stages (smem_fft);
//   two-step  -- L = R1 R2: each thread loads R2 elements straight into
//                registers, runs an R2-point DFT and one twiddle, exchanges
//                through shared memory once, runs an R1-point DFT and stores.
// GEN: L = 2^a 3^b with a radix-3 stage (a separate instantiation, so that
// the power-of-two kernels keep their registers)
template <typename T, int B, bool GEN = false>
__global__ void k_fft_xy_st(C2<T> *data, long long astride, int L, long long sj,
                            long long so, int mz, int sign, const C2<T> *twg) {
  constexpr int P = B + 1;
  constexpr int LB = clog2(B);
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *s = tw + L;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int z0 = blockIdx.x * B;
  const int bv = min(B, mz - z0);
  C2<T> *base = data + blockIdx.z * astride + (long long)blockIdx.y * so + z0;
  load_table(tw, twg, L, tid, nt);
  for (int idx = tid; idx < L * B; idx += nt) {
    const int b = idx & (B - 1), j = idx >> LB;
    s[j * P + b] = (b < bv) ? base[(long long)j * sj + b] : mk2<T>(0, 0);
  }
  __syncthreads();
  if constexpr (GEN)
    smem_fft_g<T, B, kFftK>(s, L, P, tw, sign, tid, nt);
  else
    smem_fft<T, B, kFftK>(s, L, P, tw, sign, tid, nt);
  for (int idx = tid; idx < L * B; idx += nt) {
    const int b = idx & (B - 1), j = idx >> LB;
    if (b < bv) base[(long long)j * sj + b] = s[j * P + b];
  }
}

template <typename T, int L, int B>
__global__ void __launch_bounds__(pass_threads<L, B>()) k_fft_xy_2s(C2<T> *data, long long astride, long long sj, long long so, int mz,
                         int sign, const C2<T> *twg) {
  constexpr int R1 = Fac<L>::R1, R2 = Fac<L>::R2;
  constexpr int LB = clog2(B), P = B;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *x1 = tw + L;  // [n1*R2 + k2][P]
  const int tid = threadIdx.x, nt = blockDim.x;
  const int z0 = blockIdx.x * B;
  const int bv = min(B, mz - z0);
  C2<T> *base = data + blockIdx.z * astride + (long long)blockIdx.y * so + z0;
  load_table(tw, twg, L, tid, nt);
  __syncthreads();
  if (tid < R1 * B) {
    const int b = tid & (B - 1), n1 = tid >> LB;
    C2<T> v[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2)
      v[n2] = (b < bv) ? base[(long long)(n1 + R1 * n2) * sj + b] : mk2<T>(0, 0);
    reg_dft<T, R2>(v, tw, L / R2, sign);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2)
      x1[xrow<L>(n1 * R2 + k2) * P + b] = (k2 == 0) ? v[k2] : cmul(v[k2], twid(tw, (n1 * k2) & (L - 1), sign));
  }
  __syncthreads();
  if (tid < R2 * B) {
    const int b = tid & (B - 1), k2 = tid >> LB;
    C2<T> u[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) u[n1] = x1[xrow<L>(n1 * R2 + k2) * P + b];
    reg_dft<T, R1>(u, tw, L / R1, sign);
    if (b < bv) {
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) base[(long long)(k2 + R2 * k1) * sj + b] = u[k1];
    }
  }
}

// the body of k_fft_xy_2s for the variant below
template <typename T, int L, int B>
__device__ __forceinline__ void xy_2s_body(C2<T> *data, long long astride, long long sj,
                                           long long so, int mz, int sign, const C2<T> *twg) {
  constexpr int R1 = Fac<L>::R1, R2 = Fac<L>::R2;
  constexpr int LB = clog2(B), P = B;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *x1 = tw + L;  // [n1*R2 + k2][P]
  const int tid = threadIdx.x, nt = blockDim.x;
  const int z0 = blockIdx.x * B;
  const int bv = min(B, mz - z0);
  C2<T> *base = data + blockIdx.z * astride + (long long)blockIdx.y * so + z0;
  load_table(tw, twg, L, tid, nt);
  __syncthreads();
  if (tid < R1 * B) {
    const int b = tid & (B - 1), n1 = tid >> LB;
    C2<T> v[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2)
      v[n2] = (b < bv) ? base[(long long)(n1 + R1 * n2) * sj + b] : mk2<T>(0, 0);
    reg_dft<T, R2>(v, tw, L / R2, sign);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2)
      x1[xrow<L>(n1 * R2 + k2) * P + b] = (k2 == 0) ? v[k2] : cmul(v[k2], twid(tw, (n1 * k2) & (L - 1), sign));
  }
  __syncthreads();
  if (tid < R2 * B) {
    const int b = tid & (B - 1), k2 = tid >> LB;
    C2<T> u[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) u[n1] = x1[xrow<L>(n1 * R2 + k2) * P + b];
    reg_dft<T, R1>(u, tw, L / R1, sign);
    if (b < bv) {
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) base[(long long)(k2 + R2 * k1) * sj + b] = u[k1];
    }
  }
}

// The same engine compiled for more resident CTAs (FV_TWOSTEP_HALF_OCC, FP32):
// 1280 threads per SM (10 CTAs of 128 at L = 256: at most 51 registers
// instead of the 80 the plain build takes, fewer loads in flight per warp,
// more warps); the autotuner keeps it only where it is faster.
template <int L, int B> __host__ __device__ constexpr int occ_min_blocks() {
  return 1280 / pass_threads<L, B>() > 1 ? 1280 / pass_threads<L, B>() : 1;
}
template <typename T, int L, int B>
__global__ void __launch_bounds__(pass_threads<L, B>(), (occ_min_blocks<L, B>())) k_fft_xy_2s_occ(
    C2<T> *data, long long astride, long long sj, long long so, int mz, int sign,
    const C2<T> *twg) {
  xy_2s_body<T, L, B>(data, astride, sj, so, mz, sign, twg);
}

// ---------------------------------------------------------------------------
// Three-step engine: L = R1 R2 with R2 <= 8 held per thread, and the R1-point
// DFTs of step 2 themselves split as R1 = Ra Rb, so no thread holds more than
// 8 values and twice as many warps fit on an SM as with the two-step engine.
//   step 1 : thread (b, n1) DFT_R2 over x[n1 + R1 n2], twiddle w_L^(n1 k2)
//   step 2a: thread (b, k2, m1) DFT_Rb over E1[m1 + Ra m2][k2],
//            twiddle w_R1^(m1 j2)
//   step 2b: thread (b, k2, j2) DFT_Ra over m1 -> X[k2 + R2 (j2 + Rb j1)]
// One tile buffer [L][B] (rows of one line) holds both exchanges.
template <int L> struct Fac3;
template <> struct Fac3<64> { static constexpr int R2 = 8, Ra = 2, Rb = 4; };
template <> struct Fac3<128> { static constexpr int R2 = 8, Ra = 4, Rb = 4; };
template <> struct Fac3<256> { static constexpr int R2 = 8, Ra = 4, Rb = 8; };
template <> struct Fac3<512> { static constexpr int R2 = 8, Ra = 8, Rb = 8; };
template <int L, int B> __host__ __device__ constexpr int threads3() {
  return (L / Fac3<L>::R2 > Fac3<L>::R2 * Fac3<L>::Ra ? L / Fac3<L>::R2 : Fac3<L>::R2 * Fac3<L>::Ra) *
         B;
}

template <typename T, int L, int B>
__global__ void __launch_bounds__(threads3<L, B>()) k_fft_xy_3s(C2<T> *data, long long astride, long long sj, long long so, int mz,
                         int sign, const C2<T> *twg) {
  constexpr int R2 = Fac3<L>::R2, Ra = Fac3<L>::Ra, Rb = Fac3<L>::Rb, R1 = Ra * Rb;
  constexpr int LB = clog2(B);
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *e = tw + L;  // [L][B]
  const int tid = threadIdx.x, nt = blockDim.x;
  const int z0 = blockIdx.x * B;
  const int bv = min(B, mz - z0);
  C2<T> *base = data + blockIdx.z * astride + (long long)blockIdx.y * so + z0;
  load_table(tw, twg, L, tid, nt);
  __syncthreads();
  const int b = tid & (B - 1), q = tid >> LB;
  if (q < R1) {  // step 1: q = n1
    C2<T> v[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2)
      v[n2] = (b < bv) ? base[(long long)(q + R1 * n2) * sj + b] : mk2<T>(0, 0);
    reg_dft<T, R2>(v, tw, L / R2, sign);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2)
      e[(q * R2 + k2) * B + b] = (k2 == 0) ? v[k2] : cmul(v[k2], twid(tw, (q * k2) & (L - 1), sign));
  }
  __syncthreads();
  C2<T> u[Rb];
  const int m1 = q % Ra, k2a = q / Ra;
  if (q < R2 * Ra) {  // step 2a: q = m1 + Ra k2
#pragma unroll
    for (int m2 = 0; m2 < Rb; ++m2) u[m2] = e[((m1 + Ra * m2) * R2 + k2a) * B + b];
    reg_dft<T, Rb>(u, tw, L / Rb, sign);
  }
  __syncthreads();
  if (q < R2 * Ra) {
#pragma unroll
    for (int j2 = 0; j2 < Rb; ++j2)
      e[((k2a * Rb + j2) * Ra + m1) * B + b] =
          (j2 == 0) ? u[j2] : cmul(u[j2], twid(tw, (m1 * j2 * R2) & (L - 1), sign));
  }
  __syncthreads();
  // step 2b: tasks (b, j2 + Rb k2), R2 Rb of them per pencil
  for (int task = q; task < R2 * Rb; task += nt >> LB) {
    const int j2 = task % Rb, k2 = task / Rb;
    C2<T> w[Ra];
#pragma unroll
    for (int mm = 0; mm < Ra; ++mm) w[mm] = e[((k2 * Rb + j2) * Ra + mm) * B + b];
    reg_dft<T, Ra>(w, tw, L / Ra, sign);
    if (b < bv) {
#pragma unroll
      for (int j1 = 0; j1 < Ra; ++j1) base[(long long)(k2 + R2 * (j2 + Rb * j1)) * sj + b] = w[j1];
    }
  }
}

// ---------------------------------------------------------------------------
// Pipelined two-step engine: persistent CTAs walk the tiles of the pass; the
// next tile is copied global -> shared with cp.async while the current one is
// transformed, so every CTA keeps a whole tile of loads in flight (the plain
// engines idle their loads during the arithmetic).  The tile buffer is
// [L][B] without padding -- a row is one 128-byte line (or half), so the
// line-wise accesses of both steps are free of bank conflicts -- and after
// step 1 has read it into registers it is reused for the exchange (the
// cp.async helpers are in ih_fftcore.cuh).

// tile t of a pass -> its first element and the valid pencils of the tile
struct XYTiles {
  long long astride, so;
  int mz, ntz, outer;
  template <typename V>
  __device__ __forceinline__ V *base(V *data, long long t, int B, int &bv) const {
    const int zt = (int)(t % ntz);
    const long long r = t / ntz;
    const int o = (int)(r % outer);
    const long long a = r / outer;
    const int z0 = zt * B;
    bv = min(B, mz - z0);
    return data + a * astride + (long long)o * so + z0;
  }
};

// copy tile t into buf (masked pencils zero-filled, nothing read for them)
template <typename T, int L, int B>
__device__ __forceinline__ void tile_prefetch(const C2<T> *data, const XYTiles &tl, long long t,
                                              long long sj, C2<T> *buf) {
  constexpr int LB = clog2(B);
  int bv;
  const C2<T> *base = tl.base(data, t, B, bv);
  for (int idx = threadIdx.x; idx < L * B; idx += blockDim.x) {
    const int b = idx & (B - 1), j = idx >> LB;
    const bool ok = b < bv;
    cp_async_c<T>(buf + idx, ok ? base + (long long)j * sj + b : base, ok);
  }
  cp_async_commit();
}

template <typename T, int L, int B>
__global__ void __launch_bounds__(pass_threads<L, B>(), 2) k_fft_xy_pipe(C2<T> *data, long long sj, XYTiles tl, long long total,
                                             int sign, const C2<T> *twg) {
  constexpr int R1 = Fac<L>::R1, R2 = Fac<L>::R2;
  constexpr int LB = clog2(B);
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *buf0 = tw + L;  // two tiles [L][B]
  const int tid = threadIdx.x;
  load_table(tw, twg, L, tid, blockDim.x);
  long long t = blockIdx.x;
  if (t < total) tile_prefetch<T, L, B>(data, tl, t, sj, buf0);
  const int b = tid & (B - 1), n1 = tid >> LB;
  for (int cur = 0; t < total; t += gridDim.x, cur ^= 1) {
    C2<T> *bc = buf0 + cur * L * B;
    const long long tn = t + gridDim.x;
    if (tn < total) {
      tile_prefetch<T, L, B>(data, tl, tn, sj, buf0 + (cur ^ 1) * L * B);
    } else {
      cp_async_commit();  // an empty group keeps the wait count uniform
    }
    cp_async_wait<1>();
    __syncthreads();
    C2<T> v[R2];
    if (tid < R1 * B) {
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) v[n2] = bc[(n1 + R1 * n2) * B + b];
      reg_dft<T, R2>(v, tw, L / R2, sign);
    }
    __syncthreads();
    if (tid < R1 * B) {
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2)
        bc[(n1 * R2 + k2) * B + b] = (k2 == 0) ? v[k2] : cmul(v[k2], twid(tw, (n1 * k2) & (L - 1), sign));
    }
    __syncthreads();
    if (tid < R2 * B) {
      const int k2 = tid >> LB;
      C2<T> u[R1];
#pragma unroll
      for (int m1 = 0; m1 < R1; ++m1) u[m1] = bc[(m1 * R2 + k2) * B + b];
      reg_dft<T, R1>(u, tw, L / R1, sign);
      int bv;
      C2<T> *base = tl.base(data, t, B, bv);
      if (b < bv) {
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) base[(long long)(k2 + R2 * k1) * sj + b] = u[k1];
      }
    }
    __syncthreads();  // bc is the prefetch target of the next iteration
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// z passes.  A row of H = nz/2 complex values (the real row packed as
// z_j = x_2j + i x_2j+1) belongs to a group of W = min(32, H) lanes of one
// warp; each lane holds R = H/W values in one of two index maps:
//   natural   -- lane t, register n holds element t + W n;
//   scrambled -- lane t, register k1 holds element k1 + R brev(t).
// Forward (decimation in frequency): natural in, R-point DFT in registers,
// twiddle w_H^(t k1), W-point DFT across the lanes by shuffles, scrambled out.
// Inverse (decimation in time): the mirror image, scrambled in, natural out.
// Inverse passes load their scrambled input straight from global memory (a
// row is 1-2 KB and stays in L1), so they use no shared memory; forward
// passes stage their scrambled output through a per-warp shared row so that
// whole lines are stored.
template <int H> struct ZGeo {
  static constexpr int W = H < 32 ? H : 32;
  static constexpr int R = H / W;
  static constexpr int LW = clog2(W);
  static constexpr int LR = clog2(R);
  static constexpr int G = 32 / W;  // rows per warp
  // staging row of H+1 values, swizzled within blocks of 16: element k sits
  // at k ^ ((k >> 4) & 15).  A half-warp's scrambled writes (k = k1 + R b,
  // b = brev(t)) then hit 16 distinct 8-byte bank pairs, as do its natural-
  // order reads (k = t + W n).
  static constexpr int PS = H + 16;
  __device__ static __forceinline__ int pad(int k) { return k ^ ((k >> 4) & 15); }
};

__device__ __forceinline__ int lane_brev(int t, int lw) {
  return (int)(__brev((unsigned)t) >> (32 - lw));
}

// per-lane twiddles of the forward transform (the inverse conjugates them)
template <typename T, int H> struct ZTw {
  using Gm = ZGeo<H>;
  C2<T> st[Gm::LW];  // stage q (half-span 2^q): w_(2^(q+1))^(t mod 2^q) on upper lanes, 1 on lower
  T sg[Gm::LW];      // +1 on the lower, -1 on the upper lane of stage q
  C2<T> ta[Gm::R];   // w_H^(t k1)
  __device__ __forceinline__ void load(const C2<T> *__restrict__ twh, int t) {
#pragma unroll
    for (int q = 0; q < Gm::LW; ++q) {
      const int m = 1 << q;
      const bool up = (t & m) != 0;
      sg[q] = up ? (T)-1 : (T)1;
      st[q] = up ? twh[(t & (m - 1)) * (H / (2 * m))] : mk2<T>(1, 0);
    }
#pragma unroll
    for (int k1 = 0; k1 < Gm::R; ++k1) ta[k1] = twh[t * k1];
  }
};

// natural -> scrambled, sign S
template <int S, typename T, int H>
__device__ __forceinline__ void zfft_dif(C2<T> (&v)[ZGeo<H>::R], const ZTw<T, H> &w,
                                         const C2<T> *__restrict__ twh) {
  using Gm = ZGeo<H>;
  reg_dft<T, Gm::R>(v, twh, H / Gm::R, S);
#pragma unroll
  for (int k1 = 1; k1 < Gm::R; ++k1) v[k1] = cmul(v[k1], cj<S>(w.ta[k1]));
#pragma unroll
  for (int q = Gm::LW - 1; q >= 0; --q) {
#pragma unroll
    for (int r = 0; r < Gm::R; ++r) {
      const C2<T> p = shfl_xor_c(v[r], 1 << q);
      // lower lane: v + p; upper lane: (p - v) * twiddle
      const C2<T> d = mk2<T>(fma(w.sg[q], v[r].x, p.x), fma(w.sg[q], v[r].y, p.y));
      v[r] = (q == 0) ? d : cmul(d, cj<S>(w.st[q]));
    }
  }
}

// r2c post-processing of a forward-transformed row held scrambled:
// X_k = E_k + exp(-2 pi i k/nz) O_k with E_k = (Z_k + conj Z_(H-k))/2 and
// O_k = (Z_k - conj Z_(H-k))/(2i).  v[k1] = Z_k on entry, X_k on return
// (k = k1 + R brev(t)); xH = X_H, valid on the lane with t == 0.  The partner
// Z_(H-k) of register k1 > 0 sits in register R-k1 of lane t^(W-1); that of
// register 0 in register 0 of lane brev((W - brev(t)) mod W).
// exp(-2 pi i k/nz) at the scrambled positions k = k1 + R brev(t) of lane t,
// loaded once per warp for the forward post-processing
template <typename T, int H>
__device__ __forceinline__ void zr2c_twiddles(const C2<T> *__restrict__ twz, int t,
                                              C2<T> (&wzl)[ZGeo<H>::R]) {
  using Gm = ZGeo<H>;
  const int b = lane_brev(t, Gm::LW);
#pragma unroll
  for (int k1 = 0; k1 < Gm::R; ++k1) wzl[k1] = twz[k1 + Gm::R * b];
}

template <typename T, int H>
__device__ __forceinline__ void zr2c_post_lanes(C2<T> (&v)[ZGeo<H>::R], int t, int gbase,
                                                const C2<T> (&wzl)[ZGeo<H>::R], C2<T> &xH) {
  using Gm = ZGeo<H>;
  const int b = lane_brev(t, Gm::LW);
  C2<T> pz[Gm::R];
  pz[0] = shfl_idx_c(v[0], gbase + lane_brev((Gm::W - b) & (Gm::W - 1), Gm::LW));
#pragma unroll
  for (int k1 = 1; k1 < Gm::R; ++k1) pz[k1] = shfl_xor_c(v[Gm::R - k1], Gm::W - 1);
#pragma unroll
  for (int k1 = 0; k1 < Gm::R; ++k1) {
    const C2<T> z = v[k1];
    const C2<T> zc = mk2<T>(pz[k1].x, -pz[k1].y);
    const C2<T> e = mk2<T>((T)0.5 * (z.x + zc.x), (T)0.5 * (z.y + zc.y));
    const C2<T> o = mk2<T>((T)0.5 * (z.y - zc.y), -(T)0.5 * (z.x - zc.x));
    if (k1 == 0) xH = csub(e, o);  // exp(-i pi) = -1
    v[k1] = cadd(e, cmul(o, wzl[k1]));
  }
}

// c2r input of one half-spectrum row in natural order: lane t, register n
// receives the packed Z_k = E_k + i O_k, E_k = X_k + conj X_(H-k),
// O_k = (X_k - conj X_(H-k)) exp(+2 pi i k/nz) (k = t + W n), from
// line-wise loads of X_k.
// The partner X_(H-k) is register R-1-n of lane W-t for t > 0 (one indexed
// shuffle), and lane 0's own X_0 .. X_H for t = 0.
// exp(+2 pi i k/nz) at the natural positions k = t + W n of lane t
template <typename T, int H>
__device__ __forceinline__ void zc2r_twiddles(const C2<T> *__restrict__ twz, int t,
                                              C2<T> (&wnat)[ZGeo<H>::R]) {
  using Gm = ZGeo<H>;
#pragma unroll
  for (int n = 0; n < Gm::R; ++n) {
    wnat[n] = twz[t + Gm::W * n];
    wnat[n].y = -wnat[n].y;
  }
}

template <typename T, int H>
__device__ __forceinline__ void zc2r_fetch(const C2<T> *row, int t, bool valid,
                                           C2<T> (&x)[ZGeo<H>::R], C2<T> &xH) {
  using Gm = ZGeo<H>;
#pragma unroll
  for (int n = 0; n < Gm::R; ++n) x[n] = valid ? row[t + Gm::W * n] : mk2<T>(0, 0);
  xH = (valid && t == 0) ? row[H] : mk2<T>(0, 0);
}
// the c2r pre-processing of a fetched row (element k = t + W n in register
// n of lane t, element H in xH of lane 0)
template <typename T, int H>
__device__ __forceinline__ void zc2r_prep(const C2<T> (&x)[ZGeo<H>::R], C2<T> xH, int t,
                                          int gbase, const C2<T> (&wnat)[ZGeo<H>::R],
                                          C2<T> (&z)[ZGeo<H>::R]) {
  using Gm = ZGeo<H>;
  constexpr int R = Gm::R, W = Gm::W;
  const int src = gbase + ((W - t) & (W - 1));
#pragma unroll
  for (int n = 0; n < R; ++n) {
    C2<T> pc = shfl_idx_c(x[R - 1 - n], src);
    if (t == 0) pc = (n == 0) ? xH : x[(R - n) % R];
    pc.y = -pc.y;  // conj X_(H-k)
    const C2<T> e = cadd(x[n], pc), d = csub(x[n], pc);
    const C2<T> o = cmul(d, wnat[n]);
    z[n] = mk2<T>(e.x - o.y, e.y + o.x);  // E + i O
  }
}
template <typename T, int H>
__device__ __forceinline__ void zc2r_load(const C2<T> *row, int t, int gbase, bool valid,
                                          const C2<T> (&wnat)[ZGeo<H>::R],
                                          C2<T> (&z)[ZGeo<H>::R]) {
  C2<T> x[ZGeo<H>::R], xH;
  zc2r_fetch<T, H>(row, t, valid, x, xH);
  zc2r_prep<T, H>(x, xH, t, gbase, wnat, z);
}

// a row held scrambled (register k1 of lane t = element k1 + R brev(t))
// rewritten in natural order (register n of lane t = element t + W n)
// through the warp's staging row
template <typename T, int H>
__device__ __forceinline__ void zunscramble(C2<T> (&v)[ZGeo<H>::R], int t, C2<T> *srow) {
  using Gm = ZGeo<H>;
  const int b = lane_brev(t, Gm::LW);
#pragma unroll
  for (int k1 = 0; k1 < Gm::R; ++k1) srow[Gm::pad(k1 + Gm::R * b)] = v[k1];
  __syncwarp();
#pragma unroll
  for (int n = 0; n < Gm::R; ++n) v[n] = srow[Gm::pad(t + Gm::W * n)];
  __syncwarp();
}

// store a scrambled r2c row (H+1 values) as whole lines through the warp's
// staging row
template <typename T, int H>
__device__ __forceinline__ void zstore_row(const C2<T> (&v)[ZGeo<H>::R], C2<T> xH, int t,
                                           C2<T> *srow, C2<T> *dst, bool valid) {
  using Gm = ZGeo<H>;
  const int b = lane_brev(t, Gm::LW);
#pragma unroll
  for (int k1 = 0; k1 < Gm::R; ++k1) srow[Gm::pad(k1 + Gm::R * b)] = v[k1];
  if (t == 0) srow[Gm::pad(H)] = xH;
  __syncwarp();
  if (valid) {
#pragma unroll
    for (int n = 0; n < Gm::R; ++n) dst[t + Gm::W * n] = srow[Gm::pad(t + Gm::W * n)];
    if (t == 0) dst[H] = srow[Gm::pad(H)];
  }
  __syncwarp();
}

// warps per CTA of the z passes
template <typename T> __host__ __device__ constexpr int zwarps() { return sizeof(T) == 4 ? 8 : 4; }

// forward real-to-complex pass along z: rows of nz = 2H reals -> H+1 complex
// The z-pass CTAs walk the row groups (WPB warps x G rows) with a grid
// stride, so the per-lane twiddles are loaded once per warp.
template <typename T, int H>
__global__ void __launch_bounds__(32 * zwarps<T>()) k_fft_zr2c(const T *in, long long istride, C2<T> *out, long long ostride,
                           long long rows, const C2<T> *__restrict__ twh, const C2<T> *__restrict__ twz) {
  using Gm = ZGeo<H>;
  constexpr int WPB = zwarps<T>();
  __shared__ C2<T> stage[WPB * Gm::G * Gm::PS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int t = lane & (Gm::W - 1), gi = lane >> Gm::LW;
  ZTw<T, H> w;
  w.load(twh, t);
  C2<T> wzl[Gm::R];
  zr2c_twiddles<T, H>(twz, t, wzl);
  C2<T> *srow = stage + (warp * Gm::G + gi) * Gm::PS;
  const long long ngroups = (rows + WPB * Gm::G - 1) / (WPB * Gm::G);
  for (long long rg = blockIdx.x; rg < ngroups; rg += gridDim.x) {
    const long long row = (rg * WPB + warp) * Gm::G + gi;
    const bool valid = row < rows;
    const C2<T> *src = reinterpret_cast<const C2<T> *>(in + blockIdx.y * istride) + row * H;
    C2<T> v[Gm::R];
#pragma unroll
    for (int n = 0; n < Gm::R; ++n) v[n] = valid ? src[t + Gm::W * n] : mk2<T>(0, 0);
    zfft_dif<-1, T, H>(v, w, twh);
    C2<T> xH;
    zr2c_post_lanes<T, H>(v, t, lane & ~(Gm::W - 1), wzl, xH);
    zstore_row<T, H>(v, xH, t, srow, out + blockIdx.y * ostride + row * (H + 1), valid);
  }
}

// inverse complex-to-real pass along z
template <typename T, int H>
__global__ void __launch_bounds__(32 * zwarps<T>()) k_fft_zc2r(const C2<T> *in, long long istride, T *out, long long ostride,
                           long long rows, const C2<T> *__restrict__ twh, const C2<T> *__restrict__ twz) {
  using Gm = ZGeo<H>;
  constexpr int WPB = zwarps<T>();
  __shared__ C2<T> stage[WPB * Gm::G * Gm::PS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int t = lane & (Gm::W - 1), gi = lane >> Gm::LW;
  ZTw<T, H> w;
  w.load(twh, t);
  C2<T> wnat[Gm::R];
  zc2r_twiddles<T, H>(twz, t, wnat);
  C2<T> *srow = stage + (warp * Gm::G + gi) * Gm::PS;
  const long long ngroups = (rows + WPB * Gm::G - 1) / (WPB * Gm::G);
  for (long long rg = blockIdx.x; rg < ngroups; rg += gridDim.x) {
    const long long row = (rg * WPB + warp) * Gm::G + gi;
    const bool valid = row < rows;
    C2<T> v[Gm::R];
    zc2r_load<T, H>(in + blockIdx.y * istride + row * (H + 1), t, lane & ~(Gm::W - 1), valid, wnat,
                    v);
    zfft_dif<+1, T, H>(v, w, twh);
    zunscramble<T, H>(v, t, srow);
    C2<T> *dst = reinterpret_cast<C2<T> *>(out + blockIdx.y * ostride) + row * H;
    if (valid) {
#pragma unroll
      for (int n = 0; n < Gm::R; ++n) dst[t + Gm::W * n] = v[n];
    }
  }
}


// d/dx, d/dy, d/dz and laplacian spectra of phihat/N, inverse x transform each.
// k vectors follow setup.c:609-666: first-derivative components are zero on
// the Nyquist index, k^2 keeps it.
// Two engines, as for the plain passes: Stockham (the phihat tile stays in
// shared memory for the four variants) and two-step (each step-1 thread keeps
// its R2 values of phihat in registers for the four variants).
template <typename T, int B, bool GEN = false>
__global__ void k_fft_x_deriv4_st(const C2<T> *phihat, C2<T> *out, long long ostride, Geom g,
                                   const C2<T> *twg) {
  constexpr int P = B + 1;
  constexpr int LB = clog2(B);
  extern __shared__ __align__(16) unsigned char smraw[];
  const int L = g.nx;
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *a0 = tw + L;  // phihat tile (kept)
  C2<T> *s = a0 + L * P;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int mz = g.mz;
  const int z0 = blockIdx.x * B;
  const int bv = min(B, mz - z0);
  const int yj = blockIdx.y;
  const long long sj = (long long)g.ny * mz;
  const long long off = (long long)yj * mz + z0;
  load_table(tw, twg, L, tid, nt);
  for (int idx = tid; idx < L * B; idx += nt) {
    const int b = idx & (B - 1), j = idx >> LB;
    a0[j * P + b] = (b < bv) ? phihat[off + (long long)j * sj + b] : mk2<T>(0, 0);
  }
  const int ny = g.ny, nz = g.nz, nx = g.nx;
  const T invN = (T)(1.0 / (double)g.N);
  const T fy = (2 * yj == ny) ? (T)0 : kfac<T>(g.kyu, (yj > ny / 2) ? (yj - ny) : yj);
  const int ja = (yj > ny / 2) ? (ny - yj) : yj;
  for (int a = 0; a < 4; ++a) {
    __syncthreads();
    for (int idx = tid; idx < L * B; idx += nt) {
      const int b = idx & (B - 1), i = idx >> LB;
      const int kz = z0 + b;
      C2<T> pre = a0[i * P + b];
      pre.x *= invN;
      pre.y *= invN;
      T f;
      if (a == 0) {
        f = (2 * i == nx) ? (T)0 : kfac<T>(g.kxu, (i > nx / 2) ? (i - nx) : i);
      } else if (a == 1) {
        f = fy;
      } else if (a == 2) {
        f = (2 * kz == nz) ? (T)0 : kfac<T>(g.kzu, kz);
      } else {
        f = ksq<T>(g, (i > nx / 2) ? (nx - i) : i, ja, kz);
      }
      s[i * P + b] = (a < 3) ? mk2<T>(-pre.y * f, pre.x * f)    // pre * I * k
                             : mk2<T>(-pre.x * f, -pre.y * f);  // -pre * k^2
    }
    __syncthreads();
    if constexpr (GEN)
      smem_fft_g<T, B, kFftK>(s, L, P, tw, +1, tid, nt);
    else
      smem_fft<T, B, kFftK>(s, L, P, tw, +1, tid, nt);
    C2<T> *o = out + a * ostride + off;
    for (int idx = tid; idx < L * B; idx += nt) {
      const int b = idx & (B - 1), j = idx >> LB;
      if (b < bv) o[(long long)j * sj + b] = s[j * P + b];
    }
  }
}

// the two-step fused pass keeps phihat in registers: it asks the register
// allocator for half the resident CTAs of a plain pass
template <typename T, int L, int B> __host__ __device__ constexpr int d4_min_blocks() {
  return (sizeof(T) == 4 ? 512 : 256) / pass_threads<L, B>() > 0
             ? (sizeof(T) == 4 ? 512 : 256) / pass_threads<L, B>()
             : 1;
}

template <typename T, int L, int B>
__global__ void __launch_bounds__(pass_threads<L, B>(), (d4_min_blocks<T, L, B>())) k_fft_x_deriv4_2s(const C2<T> *phihat, C2<T> *out, long long ostride, Geom g,
                                   const C2<T> *twg) {
  constexpr int R1 = Fac<L>::R1, R2 = Fac<L>::R2;
  constexpr int LB = clog2(B), P = B;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *x1 = tw + L;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int mz = g.mz;
  const int z0 = blockIdx.x * B;
  const int bv = min(B, mz - z0);
  const int yj = blockIdx.y;
  const long long sj = (long long)g.ny * mz;
  const long long off = (long long)yj * mz + z0;
  load_table(tw, twg, L, tid, nt);
  const int ny = g.ny, nz = g.nz, nx = g.nx;
  const T invN = (T)(1.0 / (double)g.N);
  const T fy = (2 * yj == ny) ? (T)0 : kfac<T>(g.kyu, (yj > ny / 2) ? (yj - ny) : yj);
  const int ja = (yj > ny / 2) ? (ny - yj) : yj;
  // step-1 threads keep their R2 values of phihat/N in registers for all four
  const bool s1 = tid < R1 * B;
  const int b1 = tid & (B - 1), n1 = tid >> LB;
  const int kz = z0 + b1;
  const T fz = (2 * kz == nz) ? (T)0 : kfac<T>(g.kzu, kz);
  C2<T> ph[R2];
#pragma unroll
  for (int n2 = 0; n2 < R2; ++n2) {
    C2<T> v = (s1 && b1 < bv) ? phihat[off + (long long)(n1 + R1 * n2) * sj + b1] : mk2<T>(0, 0);
    ph[n2] = mk2<T>(v.x * invN, v.y * invN);
  }
  for (int a = 0; a < 4; ++a) {
    __syncthreads();
    if (s1) {
      C2<T> v[R2];
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) {
        const int i = n1 + R1 * n2;
        const C2<T> pre = ph[n2];
        T f;
        if (a == 0) {
          f = (2 * i == nx) ? (T)0 : kfac<T>(g.kxu, (i > nx / 2) ? (i - nx) : i);
        } else if (a == 1) {
          f = fy;
        } else if (a == 2) {
          f = fz;
        } else {
          f = ksq<T>(g, (i > nx / 2) ? (nx - i) : i, ja, kz);
        }
        v[n2] = (a < 3) ? mk2<T>(-pre.y * f, pre.x * f)    // pre * I * k
                        : mk2<T>(-pre.x * f, -pre.y * f);  // -pre * k^2
      }
      reg_dft<T, R2>(v, tw, L / R2, +1);
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2)
        x1[xrow<L>(n1 * R2 + k2) * P + b1] = (k2 == 0) ? v[k2] : cmul(v[k2], twid(tw, (n1 * k2) & (L - 1), +1));
    }
    __syncthreads();
    if (tid < R2 * B) {
      const int b = tid & (B - 1), k2 = tid >> LB;
      C2<T> u[R1];
#pragma unroll
      for (int m1 = 0; m1 < R1; ++m1) u[m1] = x1[xrow<L>(m1 * R2 + k2) * P + b];
      reg_dft<T, R1>(u, tw, L / R1, +1);
      C2<T> *o = out + a * ostride + off;
      if (b < bv) {
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) o[(long long)(k2 + R2 * k1) * sj + b] = u[k1];
      }
    }
  }
}

// Pipelined fused x pass: persistent CTAs, the next phihat tile copied in
// with cp.async while the four variants of the current one are transformed;
// the step-1 threads keep their phihat values in registers, so the tile
// buffer doubles as the exchange buffer.
template <typename T, int L, int B>
__global__ void __launch_bounds__(pass_threads<L, B>(), 2) k_fft_x_deriv4_pipe(const C2<T> *phihat, C2<T> *out, long long ostride,
                                                   XYTiles tl, long long total, Geom g,
                                                   const C2<T> *twg) {
  constexpr int R1 = Fac<L>::R1, R2 = Fac<L>::R2;
  constexpr int LB = clog2(B);
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *buf0 = tw + L;  // two tiles [L][B]
  const int tid = threadIdx.x;
  load_table(tw, twg, L, tid, blockDim.x);
  const long long sj = (long long)g.ny * g.mz;
  const int ny = g.ny, nz = g.nz, nx = g.nx;
  const T invN = (T)(1.0 / (double)g.N);
  long long t = blockIdx.x;
  if (t < total) tile_prefetch<T, L, B>(phihat, tl, t, sj, buf0);
  const int b = tid & (B - 1), n1 = tid >> LB;
  const bool s1 = tid < R1 * B;
  for (int cur = 0; t < total; t += gridDim.x, cur ^= 1) {
    C2<T> *bc = buf0 + cur * L * B;
    const long long tn = t + gridDim.x;
    if (tn < total) {
      tile_prefetch<T, L, B>(phihat, tl, tn, sj, buf0 + (cur ^ 1) * L * B);
    } else {
      cp_async_commit();
    }
    cp_async_wait<1>();
    __syncthreads();
    // tile coordinates: y index and first z column
    const int zt = (int)(t % tl.ntz);
    const int yj = (int)((t / tl.ntz) % tl.outer);
    const int z0 = zt * B;
    const int bv = min(B, g.mz - z0);
    const long long off = (long long)yj * g.mz + z0;
    const T fy = (2 * yj == ny) ? (T)0 : kfac<T>(g.kyu, (yj > ny / 2) ? (yj - ny) : yj);
    const int ja = (yj > ny / 2) ? (ny - yj) : yj;
    const int kz = z0 + b;
    const T fz = (2 * kz == nz) ? (T)0 : kfac<T>(g.kzu, kz);
    C2<T> ph[R2];
    if (s1) {
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) {
        const C2<T> v = bc[(n1 + R1 * n2) * B + b];
        ph[n2] = mk2<T>(v.x * invN, v.y * invN);
      }
    }
    for (int a = 0; a < 4; ++a) {
      __syncthreads();  // the tile (a = 0) or the last exchange has been read
      if (s1) {
        C2<T> v[R2];
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) {
          const int i = n1 + R1 * n2;
          const C2<T> pre = ph[n2];
          T f;
          if (a == 0) {
            f = (2 * i == nx) ? (T)0 : kfac<T>(g.kxu, (i > nx / 2) ? (i - nx) : i);
          } else if (a == 1) {
            f = fy;
          } else if (a == 2) {
            f = fz;
          } else {
            f = ksq<T>(g, (i > nx / 2) ? (nx - i) : i, ja, kz);
          }
          v[n2] = (a < 3) ? mk2<T>(-pre.y * f, pre.x * f)    // pre * I * k
                          : mk2<T>(-pre.x * f, -pre.y * f);  // -pre * k^2
        }
        reg_dft<T, R2>(v, tw, L / R2, +1);
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2)
          bc[(n1 * R2 + k2) * B + b] = (k2 == 0) ? v[k2] : cmul(v[k2], twid(tw, (n1 * k2) & (L - 1), +1));
      }
      __syncthreads();
      if (tid < R2 * B) {
        const int k2 = tid >> LB;
        C2<T> u[R1];
#pragma unroll
        for (int m1 = 0; m1 < R1; ++m1) u[m1] = bc[(m1 * R2 + k2) * B + b];
        reg_dft<T, R1>(u, tw, L / R1, +1);
        C2<T> *o = out + a * ostride + off;
        if (b < bv) {
#pragma unroll
          for (int k1 = 0; k1 < R1; ++k1) o[(long long)(k2 + R2 * k1) * sj + b] = u[k1];
        }
      }
    }
    __syncthreads();  // bc is the prefetch target of the next iteration
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// z passes for any H = nz/2 = 2^a 3^b (the warp engine above needs powers of
// two): a CTA stages kZB rows in shared memory [H][kZB+1] (element j of row
// b), runs the Stockham stages along the rows and does the even/odd split of
// the real transform there (the same split as the warp engine).
constexpr int kZB = 16;
template <typename T> constexpr size_t zg_smem(int H) {
  return sizeof(C2<T>) * ((size_t)H + 2 * (size_t)H + (size_t)H * (kZB + 1));
}

template <typename T>
__global__ void k_fft_zr2c_g(const T *in, long long istride, C2<T> *out, long long ostride,
                             long long rows, int H, const C2<T> *twhg, const C2<T> *twzg) {
  constexpr int P = kZB + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *twh = reinterpret_cast<C2<T> *>(smraw);  // exp(-2 pi i k/H)
  C2<T> *twz = twh + H;                           // exp(-2 pi i k/nz)
  C2<T> *s = twz + 2 * H;
  const int tid = threadIdx.x, nt = blockDim.x;
  load_table(twh, twhg, H, tid, nt);
  load_table(twz, twzg, 2 * H, tid, nt);
  const long long r0 = (long long)blockIdx.x * kZB;
  const T *src = in + blockIdx.y * istride;
  C2<T> *dst = out + blockIdx.y * ostride;
  for (int idx = tid; idx < H * kZB; idx += nt) {  // row b, complex j = reals 2j, 2j+1
    const int j = idx % H, b = idx / H;
    const long long r = r0 + b;
    s[j * P + b] = (r < rows) ? *reinterpret_cast<const C2<T> *>(src + r * 2 * H + 2 * j)
                              : mk2<T>(0, 0);
  }
  __syncthreads();
  smem_fft_g<T, kZB, kFftK>(s, H, P, twh, -1, tid, nt);
  // X_k = E_k + exp(-2 pi i k/nz) O_k, E = (Z_k + conj Z_(H-k))/2,
  // O = (Z_k - conj Z_(H-k))/(2i), k = 0..H (Z_H = Z_0)
  for (int idx = tid; idx < (H + 1) * kZB; idx += nt) {
    const int k = idx % (H + 1), b = idx / (H + 1);
    const long long r = r0 + b;
    if (r >= rows) continue;
    const C2<T> z = s[(k % H) * P + b], zp = s[((H - k) % H) * P + b];
    const C2<T> zc = mk2<T>(zp.x, -zp.y);
    const C2<T> e = mk2<T>((T)0.5 * (z.x + zc.x), (T)0.5 * (z.y + zc.y));
    const C2<T> o = mk2<T>((T)0.5 * (z.y - zc.y), -(T)0.5 * (z.x - zc.x));
    dst[r * (H + 1) + k] = cadd(e, cmul(o, twz[k]));
  }
}

template <typename T>
__global__ void k_fft_zc2r_g(const C2<T> *in, long long istride, T *out, long long ostride,
                             long long rows, int H, const C2<T> *twhg, const C2<T> *twzg) {
  constexpr int P = kZB + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *twh = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *twz = twh + H;
  C2<T> *s = twz + 2 * H;
  const int tid = threadIdx.x, nt = blockDim.x;
  load_table(twh, twhg, H, tid, nt);
  load_table(twz, twzg, 2 * H, tid, nt);
  __syncthreads();
  const long long r0 = (long long)blockIdx.x * kZB;
  const C2<T> *src = in + blockIdx.y * istride;
  T *dst = out + blockIdx.y * ostride;
  // Z_k = E + i O, E = X_k + conj X_(H-k), O = (X_k - conj X_(H-k)) exp(+2 pi i k/nz)
  for (int idx = tid; idx < H * kZB; idx += nt) {
    const int k = idx % H, b = idx / H;
    const long long r = r0 + b;
    C2<T> zv = mk2<T>(0, 0);
    if (r < rows) {
      const C2<T> x = src[r * (H + 1) + k], xp = src[r * (H + 1) + (H - k)];
      const C2<T> pc = mk2<T>(xp.x, -xp.y);
      const C2<T> e = cadd(x, pc), d = csub(x, pc);
      C2<T> wn = twz[k];
      wn.y = -wn.y;
      const C2<T> o = cmul(d, wn);
      zv = mk2<T>(e.x - o.y, e.y + o.x);
    }
    s[k * P + b] = zv;
  }
  __syncthreads();
  smem_fft_g<T, kZB, kFftK>(s, H, P, twh, +1, tid, nt);
  for (int idx = tid; idx < H * kZB; idx += nt) {  // z_j = reals 2j, 2j+1
    const int j = idx % H, b = idx / H;
    const long long r = r0 + b;
    if (r < rows) *reinterpret_cast<C2<T> *>(dst + r * 2 * H + 2 * j) = s[j * P + b];
  }
}

// ---------------------------------------------------------------------------
// Round trip along x or y on the z spectra Z[x][y][kz] of phi.  Derivatives
// along one axis commute with the transforms along the others, so
//   out0 = scale * IFFT(i k   FFT(in))     (first derivative, 0 on Nyquist)
//   out1 = scale * IFFT(-k^2 FFT(in))      (second derivative)
// along the pencil axis give d/dx Z, d2/dx2 Z (or the y ones) without the y
// (or x) transforms; k = ku * (index folded to [-L/2, L/2)), k^2 = k2u * |index|^2
// as setup.c:609-666 defines the k vectors.
// Forward two-step: step 1 (thread b, n1) DFT_R2 over x[n1 + R1 n2] and the
// twiddle w^(-n1 k2); exchange; step 2 (thread b, k2) DFT_R1 over n1 ->
// X[k2 + R2 k1] in registers.  The inverse starts from that layout: DFT_R1
// over k1, twiddle w^(n1 k2), exchange, DFT_R2 over k2 -> x[n1 + R1 n2], the
// step-1 thread layout again.  Two exchange buffers, one per output.
// ACC (the y round trip): out1 += the second derivative + (-kz^2) in / nz,
// completing the laplacian of the x round trip; out1 and in are read again
// (in from cache) just before the last exchange, at the positions the thread
// writes.
// resident CTAs asked of the register allocator: 16 warps per SM (FP32)
template <typename T, int L, int B> __host__ __device__ constexpr int rt_min_blocks() {
  return (sizeof(T) == 4 && 512 / pass_threads<L, B>() > 1) ? 512 / pass_threads<L, B>() : 1;
}
template <typename T, int L, int B, bool ACC>
__global__ void __launch_bounds__(pass_threads<L, B>(), (rt_min_blocks<T, L, B>())) k_fft_xy_rt(
    const C2<T> *in, C2<T> *out0, C2<T> *out1, long long sj, long long so, int mz, double ku,
    double k2u, double scale, double kz2u, double invnz, const C2<T> *twg) {
  constexpr int R1 = Fac<L>::R1, R2 = Fac<L>::R2;
  constexpr int LB = clog2(B), P = B;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *e0 = tw + L;      // [L][P]
  C2<T> *e1 = e0 + L * P;  // [L][P]
  const int tid = threadIdx.x, nt = blockDim.x;
  const int z0 = blockIdx.x * B;
  const int bv = min(B, mz - z0);
  const long long off = (long long)blockIdx.y * so + z0;
  load_table(tw, twg, L, tid, nt);
  __syncthreads();
  const int b = tid & (B - 1), q = tid >> LB;
  if (q < R1) {  // q = n1
    C2<T> v[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2)
      v[n2] = (b < bv) ? in[off + (long long)(q + R1 * n2) * sj + b] : mk2<T>(0, 0);
    reg_dft<T, R2>(v, tw, L / R2, -1);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2)
      e0[xrow<L>(q * R2 + k2) * P + b] = (k2 == 0) ? v[k2] : cmul(v[k2], twid(tw, (q * k2) & (L - 1), -1));
  }
  __syncthreads();
  C2<T> u[R1];
  if (q < R2) {  // q = k2
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) u[n1] = e0[xrow<L>(n1 * R2 + q) * P + b];
  }
  __syncthreads();  // e0 is rewritten below
  if (q < R2) {
    reg_dft<T, R1>(u, tw, L / R1, -1);
    const T sc = (T)scale;
#pragma unroll
    for (int o = 0; o < 2; ++o) {
      C2<T> w[R1];
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) {
        const int k = q + R2 * k1;
        if (o == 0) {
          const T f = (2 * k == L) ? (T)0 : kfac<T>(ku, (k > L / 2) ? (k - L) : k) * sc;
          w[k1] = mk2<T>(-u[k1].y * f, u[k1].x * f);  // X * i k
        } else {
          const int ka = (k > L / 2) ? (L - k) : k;
          const T f = -((T)k2u * (T)ka * (T)ka) * sc;
          w[k1] = mk2<T>(u[k1].x * f, u[k1].y * f);  // -X k^2
        }
      }
      reg_dft<T, R1>(w, tw, L / R1, +1);
      C2<T> *e = o ? e1 : e0;
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1)
        e[xrow<L>(q * R1 + n1) * P + b] = (n1 == 0) ? w[n1] : cmul(w[n1], twid(tw, (n1 * q) & (L - 1), +1));
    }
  }
  C2<T> acc[R2];  // ACC: the x part in out1 + (-kz^2) in / nz
  if constexpr (ACC) {
    if (q < R1 && b < bv) {
      const int kz = z0 + b;
      const T f = -((T)kz2u * (T)kz * (T)kz) * (T)invnz;
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) {
        const long long i = off + (long long)(q + R1 * n2) * sj + b;
        const C2<T> zv = in[i], lx = out1[i];
        acc[n2] = mk2<T>(lx.x + f * zv.x, lx.y + f * zv.y);
      }
    }
  }
  __syncthreads();
  if (q < R1) {  // q = n1
#pragma unroll
    for (int o = 0; o < 2; ++o) {
      const C2<T> *e = o ? e1 : e0;
      C2<T> v[R2];
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) v[k2] = e[xrow<L>(k2 * R1 + q) * P + b];
      reg_dft<T, R2>(v, tw, L / R2, +1);
      C2<T> *dst = (o ? out1 : out0) + off;
      if (b < bv) {
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) {
          C2<T> r = v[n2];
          if (ACC && o == 1) r = cadd(r, acc[n2]);
          dst[(long long)(q + R1 * n2) * sj + b] = r;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Last forward pass of the tensor sources fused with update_h.  The x
// transforms of the six S_ij half spectra (after their z and y passes) of a
// tile of B pencils (one y, B consecutive kz: rows of 32 bytes) end in
// registers and go straight to the per-mode TT projection and tensor
// equation of motion (toolbox.c:311-346, 363-397): the six x-transformed
// spectra are neither written nor read back.
// Radix-4 Stockham (a radix-2 first stage when log2 L is odd), L/4 threads
// per pencil: thread j reads x[j + r L/4] (r = 0..3) from global memory,
// exchanges through shared memory between stages and ends holding
// X[j + r L/4].  A radix-4 stage of span Ns (the product of the earlier
// radices) takes data[j + r L/4] times w_L^(r (j mod Ns) L / (4 Ns)), a 4-point
// DFT, and puts the outputs at data[(j / Ns) 4 Ns + j mod Ns + r Ns].
// Buffer rows (32 bytes) are swizzled, x ^ ((x >> 2) & 3), so that every
// stage's accesses of a warp (8 threads j x B pencils) spread over the four
// 32-byte bank groups.
__device__ __forceinline__ int srow4(int x) { return x ^ ((x >> 2) & 3); }

template <typename T>
__device__ __forceinline__ void dft4_fwd(C2<T> (&v)[4]) {
  const C2<T> s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
  const C2<T> s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
  const C2<T> j13 = mk2<T>(d13.y, -d13.x);  // -i (x1 - x3)
  v[0] = cadd(s02, s13);
  v[2] = csub(s02, s13);
  v[1] = cadd(d02, j13);
  v[3] = csub(d02, j13);
}

template <typename T> __host__ __device__ constexpr int tensor_tile() {
  return 32 / (int)(2 * sizeof(T));  // pencils of a 32-byte row
}

// resident CTAs asked of the register allocator: 24 warps per SM (FP32)
template <typename T, int L, int B> __host__ __device__ constexpr int xt_min_blocks() {
  return (sizeof(T) == 4 && 768 / (L / 4 * B) > 1) ? 768 / (L / 4 * B) : 1;
}
// shared memory of k_fft_x_tensor: twiddles and two exchange buffers [L][B]
template <typename T> constexpr size_t xt_smem(int L, int B) {
  return sizeof(C2<T>) * ((size_t)L + 2 * (size_t)L * B);
}

template <typename T, int L, int B, bool NEXT>
__global__ void __launch_bounds__(L / 4 * B, (xt_min_blocks<T, L, B>())) k_fft_x_tensor(
    const C2<T> *s03, const C2<T> *s45, long long astride, T *y, T *__restrict__ out,
    const RhsScalars *rs, Geom g, const C2<T> *twg, const NextLin nl, double *outsc) {
  constexpr int Q = L / 4, LB = clog2(B);
  constexpr bool R2F = (clog2(L) & 1) != 0;
  constexpr int NS0 = R2F ? 2 : 4;                                   // span after the first stage
  constexpr int NST = L == 4 ? 0 : (clog2(Q) - clog2(NS0)) / 2 + 1;  // radix-4 stages left
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *buf = tw + L;  // two [L][B] exchange buffers
  const int tid = threadIdx.x;
  load_table(tw, twg, L, tid, Q * B);
  const int b = tid & (B - 1), j = tid >> LB;
  const int mz = g.mz, z0 = blockIdx.x * B, bv = min(B, mz - z0);
  const int yj = blockIdx.y;
  const long long sj = (long long)g.ny * mz;
  const long long off = (long long)yj * mz + z0;
  auto src_of = [&](int a) {
    return (a < 4 ? s03 + a * astride : s45 + (a - 4) * astride) + off;
  };
  C2<T> nxt[4];  // the next spectrum's inputs, loaded while this one is transformed
#pragma unroll
  for (int r = 0; r < 4; ++r)
    nxt[r] = (b < bv) ? src_of(0)[(long long)(j + r * Q) * sj + b] : mk2<T>(0, 0);
  // the thread's four modes (i = j + r L/4, yj, z0 + b): k components; the
  // projected sources accumulate spectrum by spectrum (tensor_coef)
  Mode m;
  m.j = yj;
  m.k = z0 + b;
  const int branch = (m.k != 0) ? 0 : (m.j != 0 ? 1 : 2);
  T kx[4], inv[4], ky = 0, kz = 0;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    m.i = j + r * Q;
    const ModeK<T> q = mode_k<T>(g, m);
    kx[r] = q.kx;
    ky = q.ky;
    kz = q.kz;
    inv[r] = q.ksq > (T)0 ? (T)1.0 / q.ksq : (T)0;
  }
  C2<T> n0[4], n1[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) n0[r] = n1[r] = mk2<T>(0, 0);
  int wb = 0;  // buffer of the next write
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    C2<T> v[4] = {nxt[0], nxt[1], nxt[2], nxt[3]};
    if (a + 1 < 6) {
#pragma unroll
      for (int r = 0; r < 4; ++r)
        nxt[r] = (b < bv) ? src_of(a + 1)[(long long)(j + r * Q) * sj + b] : mk2<T>(0, 0);
    }
    if constexpr (L == 4) {
      dft4_fwd<T>(v);
    } else {
      C2<T> *d = buf + wb * L * B;
      if constexpr (R2F) {  // radix 2 on (x, x + L/2) for x = j and x = j + L/4
        d[srow4(2 * j) * B + b] = cadd(v[0], v[2]);
        d[srow4(2 * j + 1) * B + b] = csub(v[0], v[2]);
        d[srow4(2 * (j + Q)) * B + b] = cadd(v[1], v[3]);
        d[srow4(2 * (j + Q) + 1) * B + b] = csub(v[1], v[3]);
      } else {
        dft4_fwd<T>(v);
#pragma unroll
        for (int r = 0; r < 4; ++r) d[srow4(4 * j + r) * B + b] = v[r];
      }
      __syncthreads();
#pragma unroll
      for (int st = 0; st < NST; ++st) {
        const int Ns = NS0 << (2 * st);
        const C2<T> *s = buf + wb * L * B;
        const int jm = j & (Ns - 1);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          v[r] = s[srow4(j + r * Q) * B + b];
          if (r > 0) v[r] = cmul(v[r], tw[r * jm * (L / (4 * Ns))]);
        }
        dft4_fwd<T>(v);
        if (st + 1 < NST) {
          wb ^= 1;
          C2<T> *d2 = buf + wb * L * B;
          const int base = (j / Ns) * 4 * Ns + jm;
#pragma unroll
          for (int r = 0; r < 4; ++r) d2[srow4(base + r * Ns) * B + b] = v[r];
          __syncthreads();
        }
      }
      wb ^= 1;  // the next spectrum writes the buffer not being read now
    }
    // v[r] = X_a[j + r L/4]
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      T al, be;
      tensor_coef<T>(a, branch, kx[r], ky, kz, kx[r] * inv[r], ky * inv[r], kz * inv[r], al, be);
      n0[r] = mk2<T>(n0[r].x + al * v[r].x, n0[r].y + al * v[r].y);
      n1[r] = mk2<T>(n1[r].x + be * v[r].x, n1[r].y + be * v[r].y);
    }
  }
  T mx = 0;
  if (b < bv) {
    const TensorConsts<T> tc(rs);
    const T dt = NEXT ? (T)*nl.dt : (T)0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      m.i = j + r * Q;
      const long long id = (long long)m.i * sj + off + b;
      const T ksq = mode_k<T>(g, m).ksq;
      const C2<T> zero = mk2<T>(0, 0);
      mx = fmax(mx, tensor_eom<T, NEXT>(g, id, id != 0 ? n0[r] : zero, id != 0 ? n1[r] : zero,
                                        id != 0 ? ksq : (T)0, tc, y, out, nl, dt));
    }
  }
  dh_max_store<T>(mx, outsc);
}


// ZSRC: the inputs are the round-trip outputs d/dx Z, d/dy Z (arrays 0, 1),
// the laplacian (array 3, completed by the y round trip) and Z itself (array
// 4), from which the z derivative is formed here.
// Otherwise arrays 0..3 hold the four full derivative spectra.
template <typename T, bool MIXED, int H, bool ZSRC>
__global__ void __launch_bounds__(32 * zwarps<T>(), (sizeof(T) == 4 && H <= 128 ? 3 : 1)) k_fft_z_rhs_fused(const C2<T> *d4, long long dstride, const T *yfl,
                                  const double *ysc, T *lap, T *pout, T *rhoout, C2<T> *s6,
                                  long long sstride4, C2<T> *s6b, int gw, double *partials,
                                  Geom g, const C2<T> *__restrict__ twh, const C2<T> *__restrict__ twz) {
  using Gm = ZGeo<H>;
  constexpr int WPB = zwarps<T>(), R = Gm::R, W = Gm::W;
  __shared__ C2<T> stage[WPB * Gm::G * Gm::PS];
  __shared__ double red[2][WPB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int t = lane & (W - 1), gi = lane >> Gm::LW;
  const long long rows = (long long)g.nx * g.ny;
  const long long row = ((long long)blockIdx.x * WPB + warp) * Gm::G + gi;
  const bool valid = row < rows;
  ZTw<T, H> w;
  w.load(twh, t);
  C2<T> *srow = stage + (warp * Gm::G + gi) * Gm::PS;
  // the four inverse transforms: d/dx, d/dy, d/dz, laplacian of phi
  C2<T> d[4][R];
  {
    C2<T> wnat[R];
    zc2r_twiddles<T, H>(twz, t, wnat);
    const T invnz = (T)(1.0 / (double)g.nz);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      C2<T> x[R], xH;
      if constexpr (ZSRC) {
        if (a == 2) {  // i kz Z / nz, zero on the Nyquist index
          C2<T> zx[R], zH;
          zc2r_fetch<T, H>(d4 + 4 * dstride + row * (H + 1), t, valid, zx, zH);
#pragma unroll
          for (int n = 0; n < R; ++n) {
            const T f = kfac<T>(g.kzu, t + W * n) * invnz;
            x[n] = mk2<T>(-zx[n].y * f, zx[n].x * f);
          }
          xH = mk2<T>(0, 0);
        } else {
          zc2r_fetch<T, H>(d4 + a * dstride + row * (H + 1), t, valid, x, xH);
        }
      } else {
        zc2r_fetch<T, H>(d4 + a * dstride + row * (H + 1), t, valid, x, xH);
      }
      zc2r_prep<T, H>(x, xH, t, lane & ~(W - 1), wnat, d[a]);
      zfft_dif<+1, T, H>(d[a], w, twh);
      zunscramble<T, H>(d[a], t, srow);
    }
  }
  // pointwise, natural map: register n holds reals 2j, 2j+1 of j = t + W n
  const long long N = g.N;
  const double a_sc = ysc[4];
  const T inv_a2 = (T)(1.0 / (a_sc * a_sc));
  const T m2 = (T)(g.mass * g.mass);
  const T third = (T)(1.0 / 3.0);
  const T phib = (T)ysc[0], pib = (T)ysc[1], psib = (T)ysc[2];
  T srho = 0, sp = 0;  // per-lane partials (2R points), then FP64
  if (valid) {
#pragma unroll
    for (int n = 0; n < R; ++n) {
      const long long e = row * (2 * H) + 2 * (t + W * n);
      const C2<T> phi = *reinterpret_cast<const C2<T> *>(yfl + e);
      const C2<T> dph = *reinterpret_cast<const C2<T> *>(yfl + N + e);
      const C2<T> ps = *reinterpret_cast<const C2<T> *>(yfl + 2 * N + e);
      C2<T> rho, p;
      rho_p<T, MIXED>(d[0][n].x, d[1][n].x, d[2][n].x, phi.x, dph.x, ps.x, inv_a2, m2, third, phib, pib,
                      psib, rho.x, p.x);
      rho_p<T, MIXED>(d[0][n].y, d[1][n].y, d[2][n].y, phi.y, dph.y, ps.y, inv_a2, m2, third, phib, pib,
                      psib, rho.y, p.y);
      *reinterpret_cast<C2<T> *>(lap + e) = d[3][n];
      *reinterpret_cast<C2<T> *>(pout + e) = p;
      if (rhoout) *reinterpret_cast<C2<T> *>(rhoout + e) = rho;
      srho += rho.x + rho.y;
      sp += p.x + p.y;
    }
  }
  // block reduction of the two sums (FP64)
  double dr = (double)srho, dp = (double)sp;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dr += __shfl_down_sync(0xffffffffu, dr, o);
    dp += __shfl_down_sync(0xffffffffu, dp, o);
  }
  if (lane == 0) {
    red[0][warp] = dr;
    red[1][warp] = dp;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0.0, sb = 0.0;
#pragma unroll
    for (int k = 0; k < WPB; ++k) {
      sa += red[0][k];
      sb += red[1][k];
    }
    partials[2 * blockIdx.x] = sa;
    partials[2 * blockIdx.x + 1] = sb;
  }
  if (!gw) return;
  // the six GW source products d_i phi d_j phi, forward transforms
  C2<T> wzl[R];
  zr2c_twiddles<T, H>(twz, t, wzl);
#pragma unroll 1
  for (int pr = 0; pr < 6; ++pr) {
    const int ia = pr < 3 ? 0 : (pr < 5 ? 1 : 2);
    const int ib = pr < 3 ? pr : (pr < 5 ? pr - 2 : 2);
    C2<T> u[R];
#pragma unroll
    for (int n = 0; n < R; ++n) {
      const C2<T> x = ia == 0 ? d[0][n] : (ia == 1 ? d[1][n] : d[2][n]);
      const C2<T> y = ib == 0 ? d[0][n] : (ib == 1 ? d[1][n] : d[2][n]);
      u[n] = mk2<T>(x.x * y.x, x.y * y.y);
    }
    zfft_dif<-1, T, H>(u, w, twh);
    C2<T> xH;
    zr2c_post_lanes<T, H>(u, t, lane & ~(W - 1), wzl, xH);
    C2<T> *dst = (pr < 4 ? s6 + pr * sstride4 : s6b + (pr - 4) * sstride4) + row * (H + 1);
    zstore_row<T, H>(u, xH, t, srow, dst, valid);
  }
}

// ---------------------------------------------------------------------------
// host launchers

// rows of a z-pass CTA
template <typename T, int H> constexpr int zrows() { return zwarps<T>() * ZGeo<H>::G; }

// CTAs of a grid-stride kernel: at most the CTAs resident on the device at
// once (the occupancy of the kernel, looked up once per kernel), at least one
static unsigned resident_grid(const void *kernel, int nt, size_t smem, int num_sms,
                              long long work) {
  static std::mutex mu;
  static std::unordered_map<const void *, int> occ_of;
  int occ = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = occ_of.find(kernel);
    if (it != occ_of.end()) {
      occ = it->second;
    } else {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, nt, smem) != cudaSuccess ||
          occ < 1)
        occ = 1;
      occ_of[kernel] = occ;
    }
  }
  const long long cap = (long long)occ * (num_sms > 0 ? num_sms : 1);
  const long long g = work < cap ? work : cap;
  return (unsigned)(g < 1 ? 1 : g);
}

template <typename T>
static const C2<T> *tab(void *p) {
  return reinterpret_cast<const C2<T> *>(p);
}


// size dispatch: calls f.template run<L>() for the power of two L
template <typename F>
static int dispatch_len(int L, F &&f, bool allow512) {
  switch (L) {
    case 4: return f.template run<4>();
    case 8: return f.template run<8>();
    case 16: return f.template run<16>();
    case 32: return f.template run<32>();
    case 64: return f.template run<64>();
    case 128: return f.template run<128>();
    case 256: return f.template run<256>();
    case 512:
      if (allow512) return f.template run<512>();
      break;
    default:
      break;
  }
  return IH_ERR_ARG;
}

// 512-point passes in both precisions (FP64 ones spill in some forms; the
// autotuner times them like the rest)
template <typename T> constexpr bool allow512() { return true; }

// threads of a Stockham tile: B*L/(4K) radix-4 butterflies, at most K each
static int threads_st(int L, int B) {
  int nt = (L * B + 4 * kFftK - 1) / (4 * kFftK);
  nt = (nt + 31) / 32 * 32;
  return nt < 64 ? 64 : nt;
}

template <typename T>
struct XYLaunch {
  Ctx *c;
  C2<T> *data;
  long long stride;
  int count, axis, sign, var;
  int cols = 0;  // columns (kz values) from data on: 0 = all mz of the plane
  int mzv() const { return cols ? cols : c->g.mz; }
  template <int B, bool GEN = false>
  int run_st(int L, dim3 grid, long long sj, long long so, const C2<T> *tw) {
    const size_t sm = sizeof(C2<T>) * ((size_t)L + (size_t)L * (B + 1));
    cudaFuncSetAttribute(k_fft_xy_st<T, B, GEN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_fft_xy_st<T, B, GEN><<<grid, threads_st(L, B), sm, c->stream>>>(data, stride, L, sj, so,
                                                                       mzv(), sign, tw);
    return IH_OK;
  }
  template <int L, int B>
  int run_2s(dim3 grid, long long sj, long long so, const C2<T> *tw) {
    const size_t sm = sizeof(C2<T>) * ((size_t)L + (size_t)L * B);
    cudaFuncSetAttribute(k_fft_xy_2s<T, L, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_xy_2s<T, L, B><<<grid, pass_threads<L, B>(), sm, c->stream>>>(data, stride, sj, so,
                                                                         mzv(), sign, tw);
    return IH_OK;
  }
  template <int L, int B>
  int run_2s_occ(dim3 grid, long long sj, long long so, const C2<T> *tw) {
    const size_t sm = sizeof(C2<T>) * ((size_t)L + (size_t)L * B);
    cudaFuncSetAttribute(k_fft_xy_2s_occ<T, L, B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_fft_xy_2s_occ<T, L, B><<<grid, pass_threads<L, B>(), sm, c->stream>>>(data, stride, sj, so,
                                                                             mzv(), sign, tw);
    return IH_OK;
  }
  template <int L, int B>
  int run_pipe(long long sj, long long so, int outer, const C2<T> *tw) {
    const Geom &g = c->g;
    const size_t sm = sizeof(C2<T>) * ((size_t)L + 2 * (size_t)L * B);
    const int nt = pass_threads<L, B>();
    static int occ = 0;  // resident CTAs per SM (a property of the kernel)
    if (!occ) {
      cudaFuncSetAttribute(k_fft_xy_pipe<T, L, B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sm);
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fft_xy_pipe<T, L, B>, nt, sm) !=
              cudaSuccess ||
          occ < 1)
        occ = 1;
    }
    XYTiles tl{stride, so, mzv(), (mzv() + B - 1) / B, outer};
    const long long total = (long long)tl.ntz * outer * count;
    const long long cap = (long long)occ * c->num_sms;
    const unsigned nb = (unsigned)(total < cap ? total : cap);
    k_fft_xy_pipe<T, L, B><<<nb, nt, sm, c->stream>>>(data, sj, tl, total, sign, tw);
    return IH_OK;
  }
  template <int L, int B>
  int run_3s(dim3 grid, long long sj, long long so, const C2<T> *tw) {
    const size_t sm = sizeof(C2<T>) * ((size_t)L + (size_t)L * B);
    cudaFuncSetAttribute(k_fft_xy_3s<T, L, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_xy_3s<T, L, B><<<grid, threads3<L, B>(), sm, c->stream>>>(data, stride, sj, so, mzv(),
                                                                     sign, tw);
    return IH_OK;
  }
  template <int L>
  int run() {
    if constexpr (L == 512 && !allow512<T>()) {
      return IH_ERR_ARG;
    } else {
      constexpr int B = tileB<T>();
      const Geom &g = c->g;
      const long long sj = axis == 0 ? (long long)g.ny * g.mz : g.mz;
      const long long so = axis == 0 ? g.mz : (long long)g.ny * g.mz;
      const int outer = axis == 0 ? g.ny : g.nx;
      const C2<T> *tw = tab<T>(axis == 0 ? c->tw_x : c->tw_y);
      if (var == FV_PIPELINED) return run_pipe<L, B>(sj, so, outer, tw);
      const int mz = mzv();
      if (var == FV_THREESTEP) {
        if constexpr (L >= 64) {
          return run_3s<L, B>(dim3((mz + B - 1) / B, outer, count), sj, so, tw);
        } else {  // short pencils: the two-step engine already holds <= 8 values
          return run_2s<L, B>(dim3((mz + B - 1) / B, outer, count), sj, so, tw);
        }
      }
      const int bw = (var == FV_TWOSTEP_HALF || var == FV_TWOSTEP_HALF_OCC) ? B / 2 : B;
      dim3 grid((mz + bw - 1) / bw, outer, count);
      if (var == FV_TWOSTEP) return run_2s<L, B>(grid, sj, so, tw);
      if (var == FV_TWOSTEP_HALF) return run_2s<L, B / 2>(grid, sj, so, tw);
      if (var == FV_TWOSTEP_HALF_OCC) {
        if constexpr (sizeof(T) == 4) {
          return run_2s_occ<L, B / 2>(grid, sj, so, tw);
        } else {  // FP64: the plain half-line engine
          return run_2s<L, B / 2>(grid, sj, so, tw);
        }
      }
      return run_st<B>(L, grid, sj, so, tw);
    }
  }
};

template <typename T>
int fft_xy(Ctx *c, C2<T> *data, long long stride, int count, int axis, int sign) {
  const Geom &g = c->g;
  const int L = axis == 0 ? g.nx : g.ny;
  prof_begin(c, KK_FFT_XY);
  if (L & (L - 1)) {  // 2^a 3^b: the Stockham engine with a radix-3 stage
    constexpr int B = tileB<T>();
    const long long sj = axis == 0 ? (long long)g.ny * g.mz : g.mz;
    const long long so = axis == 0 ? g.mz : (long long)g.ny * g.mz;
    const int outer = axis == 0 ? g.ny : g.nx;
    XYLaunch<T> xl{c, data, stride, count, axis, sign, FV_STOCKHAM};
    IH_TRY((xl.template run_st<B, true>(L, dim3((g.mz + B - 1) / B, outer, count), sj, so,
                                        tab<T>(axis == 0 ? c->tw_x : c->tw_y))));
  } else {
    IH_TRY(dispatch_len(L, XYLaunch<T>{c, data, stride, count, axis, sign, c->xy_var[axis]},
                        allow512<T>()));
  }
  prof_end(c, KK_FFT_XY, 2.0 * count * g.M * sizeof(C2<T>));
  return check_launch(c, "k_fft_xy");
}

// The forward y then x passes of the six S_ij spectra (arrays 0..3 and 5, 6
// of spec), kz slab by kz slab when w > 0: a slab of the six arrays (6 nx ny w
// complex values, 50 MB at 256^2 x 16 in FP32) stays in L2 between its y and
// its x pass, so the x pass reads it from L2 and the y pass's writes are
// overwritten there before they reach HBM.  w = 0: whole arrays (y passes,
// then x passes).  The last slab takes the remainder (w to 2w - 1 columns).
template <typename T>
int fft_gw_yx(Ctx *c, C2<T> *spec, int w) {
  const Geom &g = c->g;
  const long long M = g.M;
  if (w <= 0 || !g.pow2 || w >= g.mz) {
    IH_TRY((fft_xy<T>(c, spec, M, 4, 1, -1)));
    IH_TRY((fft_xy<T>(c, spec + 5 * M, M, 2, 1, -1)));
    IH_TRY((fft_xy<T>(c, spec, M, 4, 0, -1)));
    return fft_xy<T>(c, spec + 5 * M, M, 2, 0, -1);
  }
  const int ns = g.mz / w;
  for (int q = 0; q < ns; ++q) {
    const int z0 = q * w, ws = (q + 1 < ns) ? w : g.mz - z0;
    for (int axis = 1; axis >= 0; --axis) {
      for (int grp = 0; grp < 2; ++grp) {
        const int count = grp ? 2 : 4;
        C2<T> *d = spec + (grp ? 5 * M : 0) + z0;
        const int L = axis == 0 ? g.nx : g.ny;
        prof_begin(c, KK_FFT_XY);
        XYLaunch<T> xl{c, d, M, count, axis, -1, c->xy_var[axis]};
        xl.cols = ws;
        IH_TRY(dispatch_len(L, xl, allow512<T>()));
        prof_end(c, KK_FFT_XY, 2.0 * count * (double)g.nx * g.ny * ws * sizeof(C2<T>));
        IH_TRY(check_launch(c, "k_fft_xy"));
      }
    }
  }
  return IH_OK;
}

template <typename T>
struct ZLaunch {
  Ctx *c;
  const void *in;
  long long istride;
  void *out;
  long long ostride;
  int count;
  bool forward;
  template <int H>
  int run() {
    if constexpr (H > 256) {
      return IH_ERR_ARG;
    } else {
      constexpr int RB = zrows<T, H>();
      const Geom &g = c->g;
      const long long rows = (long long)g.nx * g.ny;
      const long long groups = (rows + RB - 1) / RB;
      const void *kf = forward ? (const void *)k_fft_zr2c<T, H> : (const void *)k_fft_zc2r<T, H>;
      dim3 grid(resident_grid(kf, 32 * zwarps<T>(), 0, c->num_sms, groups), count, 1);
      const int nt = 32 * zwarps<T>();
      if (forward) {
        k_fft_zr2c<T, H><<<grid, nt, 0, c->stream>>>((const T *)in, istride, (C2<T> *)out, ostride,
                                                     rows, tab<T>(c->tw_h), tab<T>(c->tw_z));
      } else {
        k_fft_zc2r<T, H><<<grid, nt, 0, c->stream>>>((const C2<T> *)in, istride, (T *)out, ostride,
                                                     rows, tab<T>(c->tw_h), tab<T>(c->tw_z));
      }
      return IH_OK;
    }
  }
};

template <typename T>
int fft_zr2c(Ctx *c, const T *in, long long in_stride, C2<T> *out, long long out_stride,
             int count) {
  const Geom &g = c->g;
  prof_begin(c, KK_FFT_ZR2C);
  if (fused_wide_ok(c)) {
    IH_TRY(zr2c_wide_launch(c, in, in_stride, out, out_stride, count));
  } else if (g.h & (g.h - 1)) {
    const long long rows = (long long)g.nx * g.ny;
    const size_t sm = zg_smem<T>(g.h);
    cudaFuncSetAttribute(k_fft_zr2c_g<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_zr2c_g<T><<<dim3((unsigned)((rows + kZB - 1) / kZB), count), threads_st(g.h, kZB), sm,
                      c->stream>>>(in, in_stride, out, out_stride, rows, g.h, tab<T>(c->tw_h),
                                   tab<T>(c->tw_z));
  } else {
    IH_TRY(dispatch_len(g.h, ZLaunch<T>{c, in, in_stride, out, out_stride, count, true}, false));
  }
  prof_end(c, KK_FFT_ZR2C, (double)count * (g.N * sizeof(T) + g.M * sizeof(C2<T>)));
  return check_launch(c, "k_fft_zr2c");
}

template <typename T>
int fft_zc2r(Ctx *c, const C2<T> *in, long long in_stride, T *out, long long out_stride,
             int count) {
  const Geom &g = c->g;
  prof_begin(c, KK_FFT_ZC2R);
  if (g.h & (g.h - 1)) {
    const long long rows = (long long)g.nx * g.ny;
    const size_t sm = zg_smem<T>(g.h);
    cudaFuncSetAttribute(k_fft_zc2r_g<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_zc2r_g<T><<<dim3((unsigned)((rows + kZB - 1) / kZB), count), threads_st(g.h, kZB), sm,
                      c->stream>>>(in, in_stride, out, out_stride, rows, g.h, tab<T>(c->tw_h),
                                   tab<T>(c->tw_z));
  } else {
    IH_TRY(dispatch_len(g.h, ZLaunch<T>{c, in, in_stride, out, out_stride, count, false}, false));
  }
  prof_end(c, KK_FFT_ZC2R, (double)count * (g.N * sizeof(T) + g.M * sizeof(C2<T>)));
  return check_launch(c, "k_fft_zc2r");
}

template <typename T>
int fft_r2c(Ctx *c, const T *in, long long in_stride, C2<T> *out, long long out_stride,
            int count) {
  IH_TRY(fft_zr2c<T>(c, in, in_stride, out, out_stride, count));
  IH_TRY(fft_xy<T>(c, out, out_stride, count, 1, -1));
  IH_TRY(fft_xy<T>(c, out, out_stride, count, 0, -1));
  return IH_OK;
}

template <typename T>
int fft_c2r(Ctx *c, C2<T> *in, long long in_stride, T *out, long long out_stride, int count) {
  IH_TRY(fft_xy<T>(c, in, in_stride, count, 0, +1));
  IH_TRY(fft_xy<T>(c, in, in_stride, count, 1, +1));
  IH_TRY(fft_zc2r<T>(c, in, in_stride, out, out_stride, count));
  return IH_OK;
}

template <typename T>
struct D4Launch {
  Ctx *c;
  const C2<T> *phihat;
  C2<T> *out;
  long long out_stride;
  int var;
  template <int L, int B>
  int run_2s() {
    const Geom &g = c->g;
    dim3 grid((g.mz + B - 1) / B, g.ny, 1);
    const size_t sm = sizeof(C2<T>) * ((size_t)L + (size_t)L * B);
    cudaFuncSetAttribute(k_fft_x_deriv4_2s<T, L, B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_fft_x_deriv4_2s<T, L, B><<<grid, pass_threads<L, B>(), sm, c->stream>>>(
        phihat, out, out_stride, g, tab<T>(c->tw_x));
    return IH_OK;
  }
  template <int L, int B>
  int run_pipe() {
    const Geom &g = c->g;
    const size_t sm = sizeof(C2<T>) * ((size_t)L + 2 * (size_t)L * B);
    const int nt = pass_threads<L, B>();
    static int occ = 0;
    if (!occ) {
      cudaFuncSetAttribute(k_fft_x_deriv4_pipe<T, L, B>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fft_x_deriv4_pipe<T, L, B>, nt,
                                                        sm) != cudaSuccess ||
          occ < 1)
        occ = 1;
    }
    XYTiles tl{0, g.mz, g.mz, (g.mz + B - 1) / B, g.ny};
    const long long total = (long long)tl.ntz * g.ny;
    const long long cap = (long long)occ * c->num_sms;
    const unsigned nb = (unsigned)(total < cap ? total : cap);
    k_fft_x_deriv4_pipe<T, L, B><<<nb, nt, sm, c->stream>>>(phihat, out, out_stride, tl, total, g,
                                                            tab<T>(c->tw_x));
    return IH_OK;
  }
  // the Stockham form (GEN: the only form for L = 2^a 3^b with b > 0)
  template <bool GEN = false>
  int run_st(int L) {
    constexpr int B = tileB<T>();
    const Geom &g = c->g;
    dim3 grid((g.mz + B - 1) / B, g.ny, 1);
    const size_t sm = sizeof(C2<T>) * ((size_t)L + 2 * (size_t)L * (B + 1));
    cudaFuncSetAttribute(k_fft_x_deriv4_st<T, B, GEN>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_x_deriv4_st<T, B, GEN><<<grid, threads_st(L, B), sm, c->stream>>>(
        phihat, out, out_stride, g, tab<T>(c->tw_x));
    return IH_OK;
  }
  template <int L>
  int run() {
    if constexpr (L == 512 && !allow512<T>()) {
      return IH_ERR_ARG;
    } else {
      constexpr int B = tileB<T>();
      if (var == FV_PIPELINED) return run_pipe<L, B>();
      if (var == FV_TWOSTEP) return run_2s<L, B>();
      if (var == FV_TWOSTEP_HALF) return run_2s<L, B / 2>();
      return run_st(L);
    }
  }
};

template <typename T>
int fft_x_deriv4_inv(Ctx *c, const C2<T> *phihat, C2<T> *out, long long out_stride) {
  const Geom &g = c->g;
  prof_begin(c, KK_X_DERIV4);
  if (g.nx & (g.nx - 1))
    IH_TRY((D4Launch<T>{c, phihat, out, out_stride, FV_STOCKHAM}.template run_st<true>(g.nx)));
  else
    IH_TRY(dispatch_len(g.nx, D4Launch<T>{c, phihat, out, out_stride, c->d4_var}, allow512<T>()));
  prof_end(c, KK_X_DERIV4, 5.0 * g.M * sizeof(C2<T>));
  return check_launch(c, "k_fft_x_deriv4_inv");
}

template <typename T>
struct RTLaunch {
  Ctx *c;
  const C2<T> *z;
  C2<T> *d1, *d2;
  int axis, var;
  template <int L, int B>
  int go(dim3 grid, long long sj, long long so, double ku, double k2u, double scale,
         const C2<T> *tw) {
    const size_t sm = sizeof(C2<T>) * ((size_t)L + 2 * (size_t)L * B);
    const double invnz = 1.0 / (double)c->g.nz;
    if (axis == 1) {
      cudaFuncSetAttribute(k_fft_xy_rt<T, L, B, true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      k_fft_xy_rt<T, L, B, true><<<grid, pass_threads<L, B>(), sm, c->stream>>>(
          z, d1, d2, sj, so, c->g.mz, ku, k2u, scale, c->g.kz2, invnz, tw);
    } else {
      cudaFuncSetAttribute(k_fft_xy_rt<T, L, B, false>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      k_fft_xy_rt<T, L, B, false><<<grid, pass_threads<L, B>(), sm, c->stream>>>(
          z, d1, d2, sj, so, c->g.mz, ku, k2u, scale, c->g.kz2, invnz, tw);
    }
    return IH_OK;
  }
  template <int L>
  int run() {
    if constexpr (L == 512 && !allow512<T>()) {
      return IH_ERR_ARG;
    } else {
      constexpr int B = tileB<T>();
      const Geom &g = c->g;
      const long long sj = axis == 0 ? (long long)g.ny * g.mz : g.mz;
      const long long so = axis == 0 ? g.mz : (long long)g.ny * g.mz;
      const int outer = axis == 0 ? g.ny : g.nx;
      const double ku = axis == 0 ? g.kxu : g.kyu;
      const double k2u = axis == 0 ? g.kx2 : g.ky2;
      const double scale = 1.0 / ((double)L * (double)g.nz);
      const C2<T> *tw = tab<T>(axis == 0 ? c->tw_x : c->tw_y);
      if (var == FV_TWOSTEP)
        return go<L, B>(dim3((g.mz + B - 1) / B, outer, 1), sj, so, ku, k2u, scale, tw);
      constexpr int Bh = B / 2;
      return go<L, Bh>(dim3((g.mz + Bh - 1) / Bh, outer, 1), sj, so, ku, k2u, scale, tw);
    }
  }
};

template <typename T>
struct XTLaunch {
  Ctx *c;
  const C2<T> *s03, *s45;
  T *y;
  T *out;
  double *outsc;
  const NextLin *next;
  template <int L, bool NEXT>
  void go() {
    constexpr int B = tensor_tile<T>();
    const Geom &g = c->g;
    const size_t sm = xt_smem<T>(L, B);
    cudaFuncSetAttribute(k_fft_x_tensor<T, L, B, NEXT>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    NextLin nl = next ? *next : NextLin{};
    if (!next) nl.skip_pos = c->skip_pos;
    k_fft_x_tensor<T, L, B, NEXT><<<dim3((g.mz + B - 1) / B, g.ny, 1), L / 4 * B, sm,
                                     c->stream>>>(s03, s45, g.M, y, out, c->rs, g,
                                                  tab<T>(c->tw_x), nl, outsc);
  }
  template <int L>
  int run() {
    if constexpr (L == 512 && !allow512<T>()) {
      return IH_ERR_ARG;
    } else {
      if (next)
        go<L, true>();
      else
        go<L, false>();
      return IH_OK;
    }
  }
};

template <typename T>
int fft_x_tensor(Ctx *c, const C2<T> *s03, const C2<T> *s45, T *y, T *out, double *outsc,
                 const NextLin *next) {
  const Geom &g = c->g;
  prof_begin(c, KK_X_TENSOR);
  IH_TRY(dispatch_len(g.nx, XTLaunch<T>{c, s03, s45, y, out, outsc, next}, allow512<T>()));
  prof_end(c, KK_X_TENSOR,
           6.0 * g.M * sizeof(C2<T>) +
               ((c->skip_pos ? 6.0 : 8.0) + (next ? 4.0 * (next->n + 2) : 0.0)) * g.Next * sizeof(T));
  return check_launch(c, "k_fft_x_tensor");
}

template <typename T>
int fft_xy_roundtrip(Ctx *c, const C2<T> *z, C2<T> *d1, C2<T> *d2, int axis) {
  const Geom &g = c->g;
  prof_begin(c, KK_XY_RT);
  IH_TRY(dispatch_len(axis == 0 ? g.nx : g.ny, RTLaunch<T>{c, z, d1, d2, axis, c->rt_var[axis]},
                      allow512<T>()));
  prof_end(c, KK_XY_RT, (axis == 1 ? 4.0 : 3.0) * g.M * sizeof(C2<T>));
  return check_launch(c, "k_fft_xy_rt");
}

template <typename T>
struct FusedLaunch {
  Ctx *c;
  const C2<T> *d4;
  const T *yfl;
  const double *ysc;
  T *lap, *p, *rho;
  C2<T> *s6;
  int gw;
  double *partials;
  int *nblk_out;
  int zsrc;
  template <int H, bool ZSRC>
  void launch(unsigned nblk, int nt, long long M, C2<T> *s6b) {
    if constexpr (sizeof(T) == 4) {
      k_fft_z_rhs_fused<T, true, H, ZSRC><<<nblk, nt, 0, c->stream>>>(
          d4, M, yfl, ysc, lap, p, rho, s6, M, s6b, gw, partials, c->g, tab<T>(c->tw_h),
          tab<T>(c->tw_z));
    } else {
      k_fft_z_rhs_fused<T, false, H, ZSRC><<<nblk, nt, 0, c->stream>>>(
          d4, M, yfl, ysc, lap, p, rho, s6, M, s6b, gw, partials, c->g, tab<T>(c->tw_h),
          tab<T>(c->tw_z));
    }
  }
  template <int H>
  int run() {
    if constexpr (H > 256) {
      return IH_ERR_ARG;
    } else {
      constexpr int RB = zrows<T, H>();
      const Geom &g = c->g;
      const long long rows = (long long)g.nx * g.ny;
      const unsigned nblk = (unsigned)((rows + RB - 1) / RB);
      if (2LL * nblk > c->partials_cap) {
        c->err = "grid too large for the RHS partial-sum buffer";
        return IH_ERR_ARG;
      }
      const int nt = 32 * zwarps<T>();
      const long long M = g.M;
      C2<T> *s6b = s6 + 5 * M;  // products 4 and 5 go to spec[5], spec[6]
      if (zsrc) {
        launch<H, true>(nblk, nt, M, s6b);
      } else {
        launch<H, false>(nblk, nt, M, s6b);
      }
      *nblk_out = (int)nblk;
      return IH_OK;
    }
  }
};

template <typename T>
int fft_z_rhs_fused(Ctx *c, const C2<T> *d4, const T *yfl, const double *ysc, T *lap, T *p,
                    T *rho, C2<T> *s6, int gw, double *partials, int *nblocks_out, int zsrc,
                    int plane) {
  const Geom &g = c->g;
  prof_begin(c, KK_Z_RHS_FUSED);
  if (fused_wide_ok(c)) {  // nz = 256: the wide-row engine
    IH_TRY(fused_wide_launch(c, d4, yfl, ysc, lap, p, rho, s6, gw, partials, nblocks_out, zsrc,
                             plane));
  } else {
    if (plane) {
      c->err = "plane-major tensor sources need the wide-row z pass";
      return IH_ERR_STATE;
    }
    IH_TRY(dispatch_len(
        g.h, FusedLaunch<T>{c, d4, yfl, ysc, lap, p, rho, s6, gw, partials, nblocks_out, zsrc},
        false));
  }
  prof_end(c, KK_Z_RHS_FUSED,
           (double)(4 + (gw ? 6 : 0)) * g.M * sizeof(C2<T>) +
               (double)(3 + 2 + (rho ? 1 : 0)) * g.N * sizeof(T));
  return check_launch(c, "k_fft_z_rhs_fused");
}

// twiddle tables, computed in FP64 on the host
template <typename T>
static int upload_table(Ctx *c, void **dst, int L) {
  std::vector<C2<T>> t(L > 0 ? L : 1);
  for (int k = 0; k < L; ++k) {
    double ang = kTwoPi * (double)k / (double)L;
    t[k].x = (T)cos(ang);
    t[k].y = (T)(-sin(ang));
  }
  IH_CUDA(c, cudaMalloc(dst, sizeof(C2<T>) * t.size()));
  c->dev_bytes += sizeof(C2<T>) * t.size();
  IH_CUDA(c, cudaMemcpy(*dst, t.data(), sizeof(C2<T>) * t.size(), cudaMemcpyHostToDevice));
  return IH_OK;
}

int fft_tables(Ctx *c) {
  const Geom &g = c->g;
  if (c->mixed) {
    IH_TRY(upload_table<float>(c, &c->tw_x, g.nx));
    IH_TRY(upload_table<float>(c, &c->tw_y, g.ny));
    IH_TRY(upload_table<float>(c, &c->tw_h, g.h));
    IH_TRY(upload_table<float>(c, &c->tw_z, g.nz));
  } else {
    IH_TRY(upload_table<double>(c, &c->tw_x, g.nx));
    IH_TRY(upload_table<double>(c, &c->tw_y, g.ny));
    IH_TRY(upload_table<double>(c, &c->tw_h, g.h));
    IH_TRY(upload_table<double>(c, &c->tw_z, g.nz));
  }
  return IH_OK;
}

// ---------------------------------------------------------------------------
// autotuner: every engine variant of the x/y passes (per axis, on four
// arrays, the largest batch the RHS issues) and of the fused x pass, timed
// with CUDA events on the context stream over zeroed scratch spectra; the
// fastest is kept.  Transform timing does not depend on the data.
static const char *variant_name(int v) {
  static const char *names[FV_COUNT] = {"stockham",  "two-step",   "two-step-half",
                                        "pipelined", "three-step", "two-step-half-occ"};
  return (v >= 0 && v < FV_COUNT) ? names[v] : "unknown";
}

template <typename T>
static int autotune_t(Ctx *c) {
  const Geom &g = c->g;
  const long long M = g.M;
  if (!g.pow2) {  // 2^a 3^b: one engine per pass
    c->xy_var[0] = c->xy_var[1] = c->d4_var = FV_STOCKHAM;
    c->tensor_fused = 0;
    c->tune_report =
        "grid with a radix-3 factor: Stockham x/y passes, shared-memory z passes, the "
        "full-spectrum RHS route";
    return IH_OK;
  }
  C2<T> *sp = reinterpret_cast<C2<T> *>(c->spec[0]);
  IH_CUDA(c, cudaMemsetAsync(sp, 0, sizeof(C2<T>) * 7 * (size_t)M, c->stream));
  cudaEvent_t e0, e1;
  IH_CUDA(c, cudaEventCreate(&e0));
  IH_CUDA(c, cudaEventCreate(&e1));
  const int prof = c->prof_on;
  c->prof_on = 0;
  const int reps = 3;
  char line[256];
  std::string rep;
  int st = IH_OK;
  static const char *pass_name[5] = {"x", "y", "deriv4-x", "rt-x", "rt-y"};
  int best_t = 0;
  float tbest_t = 0.f;
  // x, y, fused x, x and y round trips
  for (int pass = 0; pass < 5 && st == IH_OK; ++pass) {
    int best = -1;
    float tbest = 0.f;
    for (int v = 0; v < FV_COUNT && st == IH_OK; ++v) {
      if (pass == 2 && (v == FV_THREESTEP || v == FV_TWOSTEP_HALF_OCC))
        continue;  // the fused x pass has neither form
      if (pass > 2 && v != FV_TWOSTEP && v != FV_TWOSTEP_HALF) continue;
      if (pass < 2) {
        c->xy_var[pass] = v;
      } else if (pass == 2) {
        c->d4_var = v;
      } else {
        c->rt_var[pass - 3] = v;
      }
      float ms = 0.f;
      for (int r = 0; r <= reps && st == IH_OK; ++r) {  // r = 0: warm-up
        if (r == 1) cudaEventRecord(e0, c->stream);
        if (pass < 2)
          st = fft_xy<T>(c, sp, M, 4, pass, -1);
        else if (pass == 2)
          st = fft_x_deriv4_inv<T>(c, sp + 4 * M, sp, M);
        else
          st = fft_xy_roundtrip<T>(c, sp + 4 * M, sp + (pass - 3) * M, sp + 3 * M,
                                   pass - 3);  // the RHS's arrays: d/dx 0, d/dy 1, laplacian 3
      }
      if (st != IH_OK) break;
      cudaEventRecord(e1, c->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        c->err = "autotune: event timing failed";
        st = IH_ERR_CUDA;
        break;
      }
      ms /= reps;
      snprintf(line, sizeof line, "%s %s %.1f us; ", pass_name[pass], variant_name(v), 1e3 * ms);
      rep += line;
      if (best < 0 || ms < tbest) {
        best = v;
        tbest = ms;
      }
    }
    if (best < 0) break;
    if (pass < 2) {
      c->xy_var[pass] = best;
    } else if (pass == 2) {
      c->d4_var = best;
    } else {
      c->rt_var[pass - 3] = best;
    }
  }
  // the last x pass of the tensor sources: x passes + update_h, or fused
  // (timed on the scratch spectra with the state vectors y -> ytmp)
  for (int v = 0; v < 2 && st == IH_OK; ++v) {
    c->tensor_fused = v;
    float ms = 0.f;
    for (int r = 0; r <= reps && st == IH_OK; ++r) {
      if (r == 1) cudaEventRecord(e0, c->stream);
      st = tensor_last_pass(c, sp, c->y.fl, c->ytmp.fl, c->ytmp.sc, nullptr);
    }
    if (st != IH_OK) break;
    cudaEventRecord(e1, c->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      c->err = "autotune: event timing failed";
      st = IH_ERR_CUDA;
      break;
    }
    ms /= reps;
    snprintf(line, sizeof line, "tensor %s %.1f us; ", v ? "fused" : "separate", 1e3 * ms);
    rep += line;
    if (v == 0 || ms < tbest_t) {
      best_t = v;
      tbest_t = ms;
    }
  }
  if (st == IH_OK) c->tensor_fused = best_t;
  // the y and x passes of the six tensor sources: whole arrays or kz slabs
  // (with the separate last x pass only; the fused one takes the x pass)
  c->gw_slab = 0;
  if (st == IH_OK && !c->tensor_fused) {
    static const int widths[4] = {0, 8, 16, 32};
    float tb = 0.f;
    for (int i = 0; i < 4 && st == IH_OK; ++i) {
      if (widths[i] >= g.mz) continue;
      float ms = 0.f;
      for (int r = 0; r <= reps && st == IH_OK; ++r) {
        if (r == 1) cudaEventRecord(e0, c->stream);
        st = fft_gw_yx<T>(c, sp, widths[i]);
      }
      if (st != IH_OK) break;
      cudaEventRecord(e1, c->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        c->err = "autotune: event timing failed";
        st = IH_ERR_CUDA;
        break;
      }
      ms /= reps;
      snprintf(line, sizeof line, "gw-yx slab %d %.1f us; ", widths[i], 1e3 * ms);
      rep += line;
      if (i == 0 || ms < tb) {
        c->gw_slab = widths[i];
        tb = ms;
      }
    }
  }
  // the tensor sources' tail (y and x transforms, projection and equation of
  // motion) row by row as chosen above, against the one-pass plane
  // transforms on plane-major sources
  c->gw_plane = 0;
  if (st == IH_OK && sizeof(T) == 4 && gw_plane_ok(c)) {
    float tail[4] = {0.f, 0.f, 0.f, 0.f};
    bool planes_usable = true;
    for (int v = 0; v < 4 && st == IH_OK; ++v) {
      for (int r = 0; r <= reps && st == IH_OK; ++r) {
        if (r == 1) cudaEventRecord(e0, c->stream);
        if (v == 3) {
          st = gw_tt_plane(c, c->gwbuf);
          if (st == IH_OK) st = update_h_tt(c, c->gwbuf, c->y.fl, c->ytmp.fl, c->ytmp.sc);
          if (st != IH_OK) {  // keep the forms timed so far
            snprintf(line, sizeof line, "gw tt planes unavailable (%s); ", c->err.c_str());
            rep += line;
            cudaStreamSynchronize(c->stream);
            cudaGetLastError();
            tail[3] = -1.f;
            st = IH_OK;
            break;
          }
        } else if (v >= 1) {
          st = gw_plane_fft(c, c->gwbuf, v);
          if (st == IH_OK) st = update_h_plane(c, c->gwbuf, c->y.fl, c->ytmp.fl, c->ytmp.sc);
          if (st != IH_OK) {  // e.g. no room for a cluster of 8: keep the row passes
            snprintf(line, sizeof line, "gw planes unavailable (%s); ", c->err.c_str());
            rep += line;
            cudaStreamSynchronize(c->stream);
            cudaGetLastError();
            planes_usable = false;
            st = IH_OK;
            break;
          }
        } else if (c->gw_slab > 0 && !c->tensor_fused) {
          st = fft_gw_yx<T>(c, sp, c->gw_slab);
          if (st == IH_OK)
            st = tensor_last_pass(c, sp, c->y.fl, c->ytmp.fl, c->ytmp.sc, nullptr, true);
        } else {
          st = fft_xy<T>(c, sp, M, 4, 1, -1);
          if (st == IH_OK) st = fft_xy<T>(c, sp + 5 * M, M, 2, 1, -1);
          if (st == IH_OK) st = tensor_last_pass(c, sp, c->y.fl, c->ytmp.fl, c->ytmp.sc, nullptr);
        }
      }
      if (st != IH_OK || !planes_usable) break;
      if (tail[v] < 0.f) continue;
      cudaEventRecord(e1, c->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&tail[v], e0, e1) != cudaSuccess) {
        c->err = "autotune: event timing failed";
        st = IH_ERR_CUDA;
        break;
      }
      tail[v] /= reps;
    }
    if (st == IH_OK && planes_usable) {
      c->gw_plane = 0;
      for (int v = 1; v < 4; ++v)
        if (tail[v] >= 0.f && tail[v] < tail[c->gw_plane]) c->gw_plane = v;
      snprintf(line, sizeof line,
               "gw tail rows %.1f us, planes %.1f us, persistent planes %.1f us, "
               "projected planes %.1f us; ",
               1e3 * tail[0], 1e3 * tail[1], 1e3 * tail[2], 1e3 * tail[3]);
      rep += line;
    }
  }
  // the fused z pass (nz = 256, mixed form): wide rows, or wide rows whose
  // next input row is copied in with cp.async during the current transform
  if (st == IH_OK && sizeof(T) == 4 && g.h == 128 && c->zwide) {
    float tz[3] = {0.f, 0.f, 0.f};
    T *lap = (T *)c->rbuf[0], *pz = (T *)c->rbuf[1];
    for (int v = 1; v <= 2 && st == IH_OK; ++v) {
      c->zwide = v;
      int nblk = 0;
      for (int r = 0; r <= reps && st == IH_OK; ++r) {
        if (r == 1) cudaEventRecord(e0, c->stream);
        st = fft_z_rhs_fused<T>(c, sp, (const T *)c->y.fl, c->y.sc, lap, pz, nullptr, sp,
                                c->p.enable_gw, c->partials, &nblk, 1, 0);
      }
      if (st != IH_OK) break;
      cudaEventRecord(e1, c->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&tz[v], e0, e1) != cudaSuccess) {
        c->err = "autotune: event timing failed";
        st = IH_ERR_CUDA;
        break;
      }
      tz[v] /= reps;
    }
    if (st == IH_OK) {
      c->zwide = tz[2] < tz[1] ? 2 : 1;
      snprintf(line, sizeof line, "z pass wide %.1f us, wide+prefetch %.1f us; ", 1e3 * tz[1],
               1e3 * tz[2]);
      rep += line;
    }
  }
  c->prof_on = prof;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != IH_OK) return st;
  snprintf(line, sizeof line,
           "chosen: x %s, y %s, deriv4-x %s, rt-x %s, rt-y %s, tensor %s, gw-yx slab %d, "
           "gw planes %d, z pass %d",
           variant_name(c->xy_var[0]), variant_name(c->xy_var[1]), variant_name(c->d4_var),
           variant_name(c->rt_var[0]), variant_name(c->rt_var[1]),
           c->tensor_fused ? "fused" : "separate", c->gw_slab, c->gw_plane, c->zwide);
  c->tune_report = rep + line;
  return IH_OK;
}

int fft_autotune(Ctx *c) {
  return c->mixed ? autotune_t<float>(c) : autotune_t<double>(c);
}

#define IH_INST(T)                                                                              \
  template int fft_r2c<T>(Ctx *, const T *, long long, C2<T> *, long long, int);                \
  template int fft_c2r<T>(Ctx *, C2<T> *, long long, T *, long long, int);                      \
  template int fft_zr2c<T>(Ctx *, const T *, long long, C2<T> *, long long, int);               \
  template int fft_zc2r<T>(Ctx *, const C2<T> *, long long, T *, long long, int);               \
  template int fft_xy<T>(Ctx *, C2<T> *, long long, int, int, int);                             \
  template int fft_gw_yx<T>(Ctx *, C2<T> *, int);                                              \
  template int fft_x_deriv4_inv<T>(Ctx *, const C2<T> *, C2<T> *, long long);                   \
  template int fft_z_rhs_fused<T>(Ctx *, const C2<T> *, const T *, const double *, T *, T *,    \
                                  T *, C2<T> *, int, double *, int *, int, int);                \
  template int fft_xy_roundtrip<T>(Ctx *, const C2<T> *, C2<T> *, C2<T> *, int);              \
  template int fft_x_tensor<T>(Ctx *, const C2<T> *, const C2<T> *, T *, T *, double *,       \
                               const NextLin *);
IH_INST(float)
IH_INST(double)
#undef IH_INST

}  // namespace ih
