// ih_fftcore.cuh -- device helpers shared by the FFT translation units:
// complex arithmetic, the in-register DFT, warp shuffles of complex values,
// the k-vector factors of the derivative spectra and the pointwise energy
// density / pressure of the fused z passes.
#pragma once
#include <utility>
#include "ih_internal.cuh"

namespace ih {

__host__ __device__ constexpr int clog2(int v) { return v <= 1 ? 0 : 1 + clog2(v >> 1); }

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

// exp(-2 pi i m/16) for a compile-time m: the cosines and sines of multiples
// of pi/8 (cos pi/8, sin pi/8, sqrt(1/2)), correctly rounded in double
template <typename T>
__device__ __forceinline__ C2<T> w16(int m) {
  constexpr double c = 0.92387953251128675613, s = 0.38268343236508977173,
                   h = 0.70710678118654752440;
  // a switch (not a table) so that a constant m folds to two literals
  switch (m & 15) {
    case 0: return mk2<T>((T)1, (T)0);
    case 1: return mk2<T>((T)c, (T)-s);
    case 2: return mk2<T>((T)h, (T)-h);
    case 3: return mk2<T>((T)s, (T)-c);
    case 4: return mk2<T>((T)0, (T)-1);
    case 5: return mk2<T>((T)-s, (T)-c);
    case 6: return mk2<T>((T)-h, (T)-h);
    case 7: return mk2<T>((T)-c, (T)-s);
    case 8: return mk2<T>((T)-1, (T)0);
    case 9: return mk2<T>((T)-c, (T)s);
    case 10: return mk2<T>((T)-h, (T)h);
    case 11: return mk2<T>((T)-s, (T)c);
    case 12: return mk2<T>((T)0, (T)1);
    case 13: return mk2<T>((T)s, (T)c);
    case 14: return mk2<T>((T)h, (T)h);
    default: return mk2<T>((T)c, (T)s);
  }
}

// bit reversal of K over BITS bits, as a compile-time constant
template <int K, int BITS> struct Brev {
  static constexpr int value = ((K & 1) << (BITS - 1)) | Brev<(K >> 1), BITS - 1>::value;
};
template <int K> struct Brev<K, 0> {
  static constexpr int value = 0;
};

// v[k] <- v[brev(k)], every index a template constant (the registers are
// renamed; nothing is staged in local memory)
template <typename T, int R, int... K>
__device__ __forceinline__ void brev_permute(C2<T> (&v)[R], std::integer_sequence<int, K...>) {
  const C2<T> t[R] = {v[Brev<K, clog2(R)>::value]...};
  ((v[K] = t[K]), ...);
}

// In-register DFT of R points: v[k] <- sum_n v[n] exp(sign 2 pi i nk/R).
// Radix-2 decimation in frequency; the bit-reversed result order is undone by
// a compile-time register permutation.  Twiddles are compile-time constants
// for R <= 16, else tw[m * ts] = exp(-2 pi i m/R).
template <typename T, int R>
__device__ __forceinline__ void reg_dft(C2<T> (&v)[R], const C2<T> *tw, int ts, int sign) {
  constexpr int LOGR = clog2(R);
#pragma unroll
  for (int s = 0; s < LOGR; ++s) {
    const int len = R >> s, half = len >> 1;
#pragma unroll
    for (int st = 0; st < R; st += len) {
#pragma unroll
      for (int j = 0; j < half; ++j) {
        const C2<T> a = v[st + j], b = v[st + j + half];
        v[st + j] = cadd(a, b);
        const C2<T> d = csub(a, b);
        if (j == 0) {
          v[st + j + half] = d;
        } else if (4 * j == len) {  // exp(sign i pi/2) = sign * i
          v[st + j + half] = mk2<T>(-(T)sign * d.y, (T)sign * d.x);
        } else {
          C2<T> w = (R <= 16) ? w16<T>(j * (16 / len)) : tw[j * (R / len) * ts];
          if (sign > 0) w.y = -w.y;
          v[st + j + half] = cmul(d, w);
        }
      }
    }
  }
  brev_permute<T, R>(v, std::make_integer_sequence<int, R>{});
}

// conjugate for the inverse direction (S = +1)
template <int S, typename V>
__device__ __forceinline__ V cj(V w) {
  if (S > 0) w.y = -w.y;
  return w;
}
template <typename V>
__device__ __forceinline__ V shfl_xor_c(V v, int m) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
  return v;
}
template <typename V>
__device__ __forceinline__ V shfl_idx_c(V v, int src) {
  v.x = __shfl_sync(0xffffffffu, v.x, src);
  v.y = __shfl_sync(0xffffffffu, v.y, src);
  return v;
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

// one complex value global -> shared with cp.async (zero-filled when !valid)
template <typename T>
__device__ __forceinline__ void cp_async_c(C2<T> *s, const C2<T> *g, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  if constexpr (sizeof(T) == 4) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(g),
                 "r"(valid ? 8 : 0)
                 : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(g),
                 "r"(valid ? 16 : 0)
                 : "memory");
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// energy density and pressure at one point (toolbox.c:172-250) from the
// gradient dx, dy, dz, phi, dphi and psi.  FP64 form: full values.  Mixed form
// (MIXED): the arguments are fluctuations about the FP64 homogeneous parts
// phib, pib (= <dphi>), psib, and rho, p are the fluctuation parts, expanded
// so that no O(1) background cancels in FP32.
template <typename T, bool MIXED>
__device__ __forceinline__ void rho_p(T dx, T dy, T dz, T phi, T dph, T ps, T inv_a2, T m2, T third,
                                      T phib, T pib, T psib, T &rho, T &p) {
  T grad = dx * dx;
  grad += dy * dy;
  grad += dz * dz;
  if (!MIXED) {
    T t1 = ((T)0.5 - ps) * dph * dph;
    T t2 = ((T)0.5 + ps) * grad * inv_a2;
    T V = m2 * phi * phi * (T)0.5;
    rho = t1 + t2 + V;
    p = t1 - t2 * third - V;
  } else {
    T pif = pib + dph;
    T kin = ((T)0.5 - psib) * ((T)2.0 * pib * dph + dph * dph) - ps * pif * pif;
    T grd = ((T)0.5 + psib + ps) * grad * inv_a2;
    T pot = m2 * phib * phi + (T)0.5 * m2 * phi * phi;
    rho = kin + grd + pot;
    p = kin - grd * third - pot;
  }
}

}  // namespace ih
