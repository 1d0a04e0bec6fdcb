// ih_fft.cu -- 3D real FFTs for power-of-two grids on GB300, FP32 and FP64.
//
// Replaces the reference's FFTW calls (src/toolbox.c:806-827; plans
// src/setup.c:524-554) with FFTW's conventions: r2c is the unnormalised
// exp(-2 pi i jk/n) transform into the half spectrum [nx][ny][nz/2+1], c2r the
// unnormalised exp(+2 pi i jk/n) inverse.
//
// Structure: three passes per transform, each a kernel that stages a tile of
// pencils in shared memory and runs an in-place radix-4 (+2) Stockham FFT on
// it.  Tiles are [L][B+1] complex (pencil index innermost, one pad column
// against bank conflicts).  In the x and y passes B is one 128-byte line of
// complex values (16 for FP32, 8 for FP64), so every global row access is a
// full line; the z passes read whole contiguous rows, so their B (rows per
// CTA) is chosen for occupancy.  Lengths and tile widths are powers of two and
// all index arithmetic is shifts and masks.  The z pass treats a real row of
// length nz as nz/2 complex values and applies the even/odd split.  Twiddles
// come from tables computed once in FP64 on the host (exp(-2 pi i k/L)) and
// staged into shared memory.
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
#include "ih_internal.cuh"

namespace ih {

template <typename T>
__device__ __forceinline__ C2<T> mk2(T x, T y) {
  C2<T> r;
  r.x = x;
  r.y = y;
  return r;
}
// complex helpers, templated on the vector type so that float2/double2 deduce
template <typename V>
__device__ __forceinline__ V cmul(V a, V b) {
  V r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename V>
__device__ __forceinline__ V cadd(V a, V b) {
  V r;
  r.x = a.x + b.x;
  r.y = a.y + b.y;
  return r;
}
template <typename V>
__device__ __forceinline__ V csub(V a, V b) {
  V r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}

template <typename T> __host__ __device__ constexpr int tileB() { return 128 / (int)(2 * sizeof(T)); }
__host__ __device__ constexpr int clog2(int v) { return v <= 1 ? 0 : 1 + clog2(v >> 1); }
static int ilog2(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

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

template <typename V>
__device__ __forceinline__ void load_table(V *dst, const V *src, int n, int tid, int nt) {
  for (int i = tid; i < n; i += nt) dst[i] = src[i];
}

// ---------------------------------------------------------------------------
// complex pass along x (axis 0) or y (axis 1), in place, batched over arrays
template <typename T>
__global__ void k_fft_xy(C2<T> *data, long long astride, int L, long long sj,
                         long long so, int mz, int sign, const C2<T> *twg) {
  constexpr int B = tileB<T>();
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
  smem_fft<T, B, kFftK>(s, L, P, tw, sign, tid, nt);
  for (int idx = tid; idx < L * B; idx += nt) {
    const int b = idx & (B - 1), j = idx >> LB;
    if (b < bv) base[(long long)j * sj + b] = s[j * P + b];
  }
}

// post-processing of one forward half-length row: X_k = E_k + w^k O_k
template <typename T>
__device__ __forceinline__ C2<T> zr2c_post(const C2<T> *s, int k, int h, int P, int b,
                                           const C2<T> *wz) {
  C2<T> z = s[(k & (h - 1)) * P + b], zc = s[((h - k) & (h - 1)) * P + b];
  zc.y = -zc.y;
  C2<T> e = mk2<T>((T)0.5 * (z.x + zc.x), (T)0.5 * (z.y + zc.y));
  // O = (Z - conj Z_{h-k}) / (2i)
  C2<T> o = mk2<T>((T)0.5 * (z.y - zc.y), -(T)0.5 * (z.x - zc.x));
  return cadd(e, cmul(o, wz[k]));
}

// forward real-to-complex pass along z: BZ rows of nz reals -> nz/2+1 complex
template <typename T, int BZ>
__global__ void k_fft_zr2c(const T *in, long long istride, C2<T> *out, long long ostride,
                           long long rows, int h, int logh, const C2<T> *twh,
                           const C2<T> *twz) {
  constexpr int P = BZ + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *wz = tw + h;
  C2<T> *s = wz + h + 1;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int mz = h + 1;
  const long long r0 = (long long)blockIdx.x * BZ;
  const int bv = (int)min((long long)BZ, rows - r0);
  const C2<T> *src = reinterpret_cast<const C2<T> *>(in + blockIdx.z * istride) + r0 * h;
  C2<T> *dst = out + blockIdx.z * ostride + r0 * mz;
  load_table(tw, twh, h, tid, nt);
  load_table(wz, twz, h + 1, tid, nt);
  for (int idx = tid; idx < BZ * h; idx += nt) {
    const int b = idx >> logh, j = idx & (h - 1);
    s[j * P + b] = (b < bv) ? src[(long long)b * h + j] : mk2<T>(0, 0);
  }
  __syncthreads();
  smem_fft<T, BZ, kFftK>(s, h, P, tw, -1, tid, nt);
  for (int b = 0; b < bv; ++b)
    for (int k = tid; k < mz; k += nt) dst[(long long)b * mz + k] = zr2c_post<T>(s, k, h, P, b, wz);
}

// z pre-processing of one half-spectrum row into the packed complex row
template <typename T>
__device__ __forceinline__ C2<T> zc2r_pre(const C2<T> *row, int k, int h, const C2<T> *wz) {
  C2<T> x = row[k], xc = row[h - k];
  xc.y = -xc.y;
  C2<T> e = cadd(x, xc), d = csub(x, xc);
  C2<T> w = wz[k];
  w.y = -w.y;  // exp(+2 pi i k / nz)
  C2<T> o = cmul(d, w);
  return mk2<T>(e.x - o.y, e.y + o.x);  // E + i O
}

// inverse complex-to-real pass along z
template <typename T, int BZ>
__global__ void k_fft_zc2r(const C2<T> *in, long long istride, T *out, long long ostride,
                           long long rows, int h, int logh, const C2<T> *twh,
                           const C2<T> *twz) {
  constexpr int P = BZ + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *wz = tw + h;
  C2<T> *s = wz + h + 1;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int mz = h + 1;
  const long long r0 = (long long)blockIdx.x * BZ;
  const int bv = (int)min((long long)BZ, rows - r0);
  const C2<T> *src = in + blockIdx.z * istride + r0 * mz;
  C2<T> *dst = reinterpret_cast<C2<T> *>(out + blockIdx.z * ostride) + r0 * h;
  load_table(tw, twh, h, tid, nt);
  load_table(wz, twz, h + 1, tid, nt);
  __syncthreads();
  for (int idx = tid; idx < BZ * h; idx += nt) {
    const int b = idx >> logh, k = idx & (h - 1);
    s[k * P + b] = (b < bv) ? zc2r_pre<T>(src + (long long)b * mz, k, h, wz) : mk2<T>(0, 0);
  }
  __syncthreads();
  smem_fft<T, BZ, kFftK>(s, h, P, tw, +1, tid, nt);
  for (int idx = tid; idx < BZ * h; idx += nt) {
    const int b = idx >> logh, j = idx & (h - 1);
    if (b < bv) dst[(long long)b * h + j] = s[j * P + b];
  }
}

// k components (setup.c:609-666).  FP64: the reference's expressions
// (pars.x.k * i; k2 = pars.z.k2*k*k + pars.x.k2*i*i + pars.y.k2*j*j).
// FP32: the same products in single precision.
template <typename T>
__device__ __forceinline__ T kfac(double unit, int n) {
  if constexpr (sizeof(T) == 8) {
    return unit * n;
  } else {
    return (float)unit * (float)n;
  }
}
template <typename T>
__device__ __forceinline__ T ksq(const Geom &g, int ia, int ja, int kz) {
  if constexpr (sizeof(T) == 8) {
    double q = g.kz2 * kz * kz;
    q += g.kx2 * ia * ia;
    q += g.ky2 * ja * ja;
    return q;
  } else {
    float q = (float)g.kz2 * (float)kz * (float)kz;
    q += (float)g.kx2 * (float)ia * (float)ia;
    q += (float)g.ky2 * (float)ja * (float)ja;
    return q;
  }
}

// d/dx, d/dy, d/dz and laplacian spectra of phihat/N, inverse x transform each.
// k vectors follow setup.c:609-666: first-derivative components are zero on
// the Nyquist index, k^2 keeps it.
template <typename T>
__global__ void k_fft_x_deriv4_inv(const C2<T> *phihat, C2<T> *out, long long ostride, Geom g,
                                   const C2<T> *twg) {
  constexpr int B = tileB<T>();
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
    smem_fft<T, B, kFftK>(s, L, P, tw, +1, tid, nt);
    C2<T> *o = out + a * ostride + off;
    for (int idx = tid; idx < L * B; idx += nt) {
      const int b = idx & (B - 1), j = idx >> LB;
      if (b < bv) o[(long long)j * sj + b] = s[j * P + b];
    }
  }
}

// The fused last inverse z pass of the RHS (see the file comment).
// Plain form (MIXED=false): the reference's expressions (toolbox.c:196-208,
// 225-243) on full values.  Mixed form: homogeneous parts in FP64 scalars,
// fluctuation parts in T:
//   rho = rho_bar + drho,  rho_bar = (1/2 - psib) Pib^2 + m^2 phib^2 / 2,
//   drho = (1/2 - psib)(2 Pib dPi + dPi^2) - dpsi (Pib + dPi)^2
//          + (1/2 + psi) g / a^2 + m^2 phib dphi + m^2 dphi^2 / 2,
// and likewise p; lap and p written as fluctuations.
template <typename T, bool MIXED, int BZ>
__global__ void k_fft_z_rhs_fused(const C2<T> *d4, long long dstride, const T *yfl,
                                  const double *ysc, T *lap, T *pout, T *rhoout, C2<T> *s6,
                                  long long sstride4, C2<T> *s6b, int gw, double *partials,
                                  Geom g, int logh, const C2<T> *twh, const C2<T> *twz) {
  constexpr int P = BZ + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int h = g.h, mz = g.mz, nz = g.nz;
  const int lognz = logh + 1;
  C2<T> *tw = reinterpret_cast<C2<T> *>(smraw);
  C2<T> *wz = tw + h;
  C2<T> *tile = wz + h + 1;  // 6 tiles of h*P
  const int TS = h * P;
  __shared__ double red[2][32];
  const int tid = threadIdx.x, nt = blockDim.x;
  const long long rows = (long long)g.nx * g.ny;
  const long long r0 = (long long)blockIdx.x * BZ;
  const int bv = (int)min((long long)BZ, rows - r0);
  load_table(tw, twh, h, tid, nt);
  load_table(wz, twz, h + 1, tid, nt);
  __syncthreads();
  for (int a = 0; a < 4; ++a) {
    const C2<T> *src = d4 + a * dstride + r0 * mz;
    C2<T> *s = tile + a * TS;
    for (int idx = tid; idx < BZ * h; idx += nt) {
      const int b = idx >> logh, k = idx & (h - 1);
      s[k * P + b] = (b < bv) ? zc2r_pre<T>(src + (long long)b * mz, k, h, wz) : mk2<T>(0, 0);
    }
  }
  __syncthreads();
  for (int a = 0; a < 4; ++a) smem_fft<T, BZ, kFftK>(tile + a * TS, h, P, tw, +1, tid, nt);
  // pointwise
  const long long N = g.N;
  const double a_sc = ysc[4];
  const T inv_a2 = (T)(1.0 / (a_sc * a_sc));
  const T m2 = (T)(g.mass * g.mass);
  const T third = (T)(1.0 / 3.0);
  T srho = 0, sp = 0;  // per-thread partials (a few points), then FP64
  T *tl = reinterpret_cast<T *>(tile);
  for (int idx = tid; idx < BZ * nz; idx += nt) {
    const int b = idx >> lognz, zi = idx & (nz - 1);
    if (b >= bv) continue;
    const int e = ((zi >> 1) * P + b) * 2 + (zi & 1);  // scalar index in a tile
    T dx = tl[e], dy = tl[2 * TS + e], dz = tl[4 * TS + e], lp = tl[6 * TS + e];
    const long long gi = (r0 + b) * nz + zi;
    T phi = yfl[gi], dph = yfl[N + gi], ps = yfl[2 * N + gi];
    T grad = dx * dx;
    grad += dy * dy;
    grad += dz * dz;
    T rho, p;
    if (!MIXED) {
      T t1 = ((T)0.5 - ps) * dph * dph;
      T t2 = ((T)0.5 + ps) * grad * inv_a2;
      T V = m2 * phi * phi * (T)0.5;
      rho = t1 + t2 + V;
      p = t1 - t2 * third - V;
    } else {
      const T phib = (T)ysc[0], pib = (T)ysc[1], psib = (T)ysc[2];
      T pif = pib + dph;
      T kin = ((T)0.5 - psib) * ((T)2.0 * pib * dph + dph * dph) - ps * pif * pif;
      T grd = ((T)0.5 + psib + ps) * grad * inv_a2;
      T pot = m2 * phib * phi + (T)0.5 * m2 * phi * phi;
      rho = kin + grd + pot;
      p = kin - grd * third - pot;
    }
    lap[gi] = lp;
    pout[gi] = p;
    if (rhoout) rhoout[gi] = rho;
    srho += rho;
    sp += p;
    if (gw) {
      // in place: the same thread owns this point in every tile
      tl[e] = dx * dx;
      tl[2 * TS + e] = dx * dy;
      tl[4 * TS + e] = dx * dz;
      tl[6 * TS + e] = dy * dy;
      tl[8 * TS + e] = dy * dz;
      tl[10 * TS + e] = dz * dz;
    }
  }
  // block reduction of the two sums (FP64)
  double dr = (double)srho, dp = (double)sp;
  for (int o = 16; o > 0; o >>= 1) {
    dr += __shfl_down_sync(0xffffffffu, dr, o);
    dp += __shfl_down_sync(0xffffffffu, dp, o);
  }
  const int lane = tid & 31, wid = tid >> 5;
  if (lane == 0) {
    red[0][wid] = dr;
    red[1][wid] = dp;
  }
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (nt + 31) / 32; ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
  }
  if (!gw) return;
  for (int a = 0; a < 6; ++a) smem_fft<T, BZ, kFftK>(tile + a * TS, h, P, tw, -1, tid, nt);
  for (int a = 0; a < 6; ++a) {
    C2<T> *dst = (a < 4 ? s6 + a * sstride4 : s6b + (a - 4) * sstride4) + r0 * mz;
    const C2<T> *s = tile + a * TS;
    for (int b = 0; b < bv; ++b)
      for (int k = tid; k < mz; k += nt) dst[(long long)b * mz + k] = zr2c_post<T>(s, k, h, P, b, wz);
  }
}

// ---------------------------------------------------------------------------
// host launchers
// threads for a tile of B pencils of length L: B*L/(4K) radix-4 butterflies
// per stage, at most K per thread
static int threads_for(int L, int B) {
  int nt = (L * B + 4 * kFftK - 1) / (4 * kFftK);
  nt = (nt + 31) / 32 * 32;
  if (nt < 64) nt = 64;
  return nt;
}

// rows per CTA of the z passes, and of the fused z pass (6 tiles)
template <typename T> constexpr int zrows() { return 8; }
template <typename T> constexpr int zrows_fused() { return sizeof(T) == 4 ? 8 : 4; }

template <typename T>
static const C2<T> *tab(void *p) {
  return reinterpret_cast<const C2<T> *>(p);
}

template <typename T>
int fft_xy(Ctx *c, C2<T> *data, long long stride, int count, int axis, int sign) {
  constexpr int B = tileB<T>();
  const Geom &g = c->g;
  const int L = axis == 0 ? g.nx : g.ny;
  const long long sj = axis == 0 ? (long long)g.ny * g.mz : g.mz;
  const long long so = axis == 0 ? g.mz : (long long)g.ny * g.mz;
  const int outer = axis == 0 ? g.ny : g.nx;
  dim3 grid((g.mz + B - 1) / B, outer, count);
  const int nt = threads_for(L, B);
  size_t sm = sizeof(C2<T>) * ((size_t)L + (size_t)L * (B + 1));
  cudaFuncSetAttribute(k_fft_xy<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  prof_begin(c, KK_FFT_XY);
  k_fft_xy<T><<<grid, nt, sm, c->stream>>>(data, stride, L, sj, so, g.mz, sign,
                                             tab<T>(axis == 0 ? c->tw_x : c->tw_y));
  prof_end(c, KK_FFT_XY, 2.0 * count * g.M * sizeof(C2<T>));
  return check_launch(c, "k_fft_xy");
}

template <typename T>
int fft_zr2c(Ctx *c, const T *in, long long in_stride, C2<T> *out, long long out_stride,
             int count) {
  constexpr int BZ = zrows<T>();
  const Geom &g = c->g;
  const long long rows = (long long)g.nx * g.ny;
  dim3 grid((unsigned)((rows + BZ - 1) / BZ), 1, count);
  const int nt = threads_for(g.h, BZ);
  size_t sm = sizeof(C2<T>) * ((size_t)2 * g.h + 1 + (size_t)g.h * (BZ + 1));
  cudaFuncSetAttribute(k_fft_zr2c<T, BZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  prof_begin(c, KK_FFT_ZR2C);
  k_fft_zr2c<T, BZ><<<grid, nt, sm, c->stream>>>(in, in_stride, out, out_stride, rows, g.h,
                                                   ilog2(g.h), tab<T>(c->tw_h), tab<T>(c->tw_z));
  prof_end(c, KK_FFT_ZR2C, (double)count * (g.N * sizeof(T) + g.M * sizeof(C2<T>)));
  return check_launch(c, "k_fft_zr2c");
}

template <typename T>
int fft_zc2r(Ctx *c, const C2<T> *in, long long in_stride, T *out, long long out_stride,
             int count) {
  constexpr int BZ = zrows<T>();
  const Geom &g = c->g;
  const long long rows = (long long)g.nx * g.ny;
  dim3 grid((unsigned)((rows + BZ - 1) / BZ), 1, count);
  const int nt = threads_for(g.h, BZ);
  size_t sm = sizeof(C2<T>) * ((size_t)2 * g.h + 1 + (size_t)g.h * (BZ + 1));
  cudaFuncSetAttribute(k_fft_zc2r<T, BZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  prof_begin(c, KK_FFT_ZC2R);
  k_fft_zc2r<T, BZ><<<grid, nt, sm, c->stream>>>(in, in_stride, out, out_stride, rows, g.h,
                                                   ilog2(g.h), tab<T>(c->tw_h), tab<T>(c->tw_z));
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
int fft_x_deriv4_inv(Ctx *c, const C2<T> *phihat, C2<T> *out, long long out_stride) {
  constexpr int B = tileB<T>();
  const Geom &g = c->g;
  dim3 grid((g.mz + B - 1) / B, g.ny, 1);
  const int nt = threads_for(g.nx, B);
  size_t sm = sizeof(C2<T>) * ((size_t)g.nx + 2 * (size_t)g.nx * (B + 1));
  cudaFuncSetAttribute(k_fft_x_deriv4_inv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  prof_begin(c, KK_X_DERIV4);
  k_fft_x_deriv4_inv<T><<<grid, nt, sm, c->stream>>>(phihat, out, out_stride, g, tab<T>(c->tw_x));
  prof_end(c, KK_X_DERIV4, 5.0 * g.M * sizeof(C2<T>));
  return check_launch(c, "k_fft_x_deriv4_inv");
}

template <typename T>
int fft_z_rhs_fused(Ctx *c, const C2<T> *d4, const T *yfl, const double *ysc, T *lap, T *p,
                    T *rho, C2<T> *s6, int gw, double *partials, int *nblocks_out) {
  constexpr int BZ = zrows_fused<T>();
  const Geom &g = c->g;
  const long long rows = (long long)g.nx * g.ny;
  const unsigned nblk = (unsigned)((rows + BZ - 1) / BZ);
  if (2LL * nblk > c->partials_cap) {
    c->err = "grid too large for the RHS partial-sum buffer";
    return IH_ERR_ARG;
  }
  int nt = threads_for(g.h, BZ);
  if (nt < 256) nt = 256;
  size_t sm = sizeof(C2<T>) * ((size_t)2 * g.h + 1 + 6 * (size_t)g.h * (BZ + 1));
  const long long M = g.M;
  C2<T> *s6b = s6 + 5 * M;  // products 4 and 5 go to spec[5], spec[6]
  const int logh = ilog2(g.h);
  prof_begin(c, KK_Z_RHS_FUSED);
  if (c->mixed) {
    cudaFuncSetAttribute(k_fft_z_rhs_fused<T, true, BZ>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_z_rhs_fused<T, true, BZ><<<nblk, nt, sm, c->stream>>>(
        d4, M, yfl, ysc, lap, p, rho, s6, M, s6b, gw, partials, g, logh, tab<T>(c->tw_h),
        tab<T>(c->tw_z));
  } else {
    cudaFuncSetAttribute(k_fft_z_rhs_fused<T, false, BZ>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_z_rhs_fused<T, false, BZ><<<nblk, nt, sm, c->stream>>>(
        d4, M, yfl, ysc, lap, p, rho, s6, M, s6b, gw, partials, g, logh, tab<T>(c->tw_h),
        tab<T>(c->tw_z));
  }
  prof_end(c, KK_Z_RHS_FUSED,
           (double)(4 + (gw ? 6 : 0)) * M * sizeof(C2<T>) +
               (double)(3 + 2 + (rho ? 1 : 0)) * g.N * sizeof(T));
  *nblocks_out = (int)nblk;
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

#define IH_INST(T)                                                                              \
  template int fft_r2c<T>(Ctx *, const T *, long long, C2<T> *, long long, int);                \
  template int fft_c2r<T>(Ctx *, C2<T> *, long long, T *, long long, int);                      \
  template int fft_zr2c<T>(Ctx *, const T *, long long, C2<T> *, long long, int);               \
  template int fft_zc2r<T>(Ctx *, const C2<T> *, long long, T *, long long, int);               \
  template int fft_xy<T>(Ctx *, C2<T> *, long long, int, int, int);                             \
  template int fft_x_deriv4_inv<T>(Ctx *, const C2<T> *, C2<T> *, long long);                   \
  template int fft_z_rhs_fused<T>(Ctx *, const C2<T> *, const T *, const double *, T *, T *,    \
                                  T *, C2<T> *, int, double *, int *);
IH_INST(float)
IH_INST(double)
#undef IH_INST

}  // namespace ih
