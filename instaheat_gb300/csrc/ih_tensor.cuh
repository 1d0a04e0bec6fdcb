// ih_tensor.cuh -- mode indexing, k vectors and the per-mode tensor update
// (TT projection of the six S_ij spectra and the equation of motion of the
// two polarisations, toolbox.c:311-346, 363-397), shared by the stand-alone
// update_h kernel and the x pass that fuses it.
#pragma once
#include "ih_internal.cuh"

namespace ih {

template <typename T>
__device__ __forceinline__ C2<T> mk2c(T x, T y) {
  C2<T> r;
  r.x = x;
  r.y = y;
  return r;
}

// mode index -> (i, j, k) of the half spectrum
struct Mode {
  int i, j, k;
};
__device__ __forceinline__ Mode mode_of(long long id, const Geom &g) {
  Mode m;
  m.k = (int)(id % g.mz);
  long long r = id / g.mz;
  m.j = (int)(r % g.ny);
  m.i = (int)(r / g.ny);
  return m;
}
// FP64 k components with the reference's Nyquist conventions
__device__ __forceinline__ double kxf_of(const Geom &g, int i) {
  return g.kxu * ((i > g.nx / 2) ? (i - g.nx) : i);
}
__device__ __forceinline__ double kyf_of(const Geom &g, int j) {
  return g.kyu * ((j > g.ny / 2) ? (j - g.ny) : j);
}
__device__ __forceinline__ double kzf_of(const Geom &g, int k) { return g.kzu * k; }
__device__ __forceinline__ double kz_deriv(const Geom &g, int k) {
  return (2 * k == g.nz) ? 0.0 : g.kzu * k;
}
// |k|^2 with the reference's operations in its order and no fused
// multiply-adds (setup.c:609-666, compiled without contraction): the same
// roundings as the C code, so that modes on a shell boundary of the spectra
// (bins |k| / k_max an integer, e.g. the grid corners) fall into the same bin
__device__ __forceinline__ double ksq64(const Geom &g, int i, int j, int k) {
  const int ia = (i > g.nx / 2) ? (g.nx - i) : i;
  const int ja = (j > g.ny / 2) ? (g.ny - j) : j;
  double q = __dmul_rn(__dmul_rn(g.kz2, (double)k), (double)k);
  q = __dadd_rn(q, __dmul_rn(__dmul_rn(g.kx2, (double)ia), (double)ia));
  q = __dadd_rn(q, __dmul_rn(__dmul_rn(g.ky2, (double)ja), (double)ja));
  return q;
}

// the RHS scalars the tensor equation of motion uses, in T
template <typename T> struct TensorConsts {
  T inv_a2, two_inv_a2, h3, pm2;
  __device__ __forceinline__ explicit TensorConsts(const RhsScalars *rs)
      : inv_a2((T)(1.0 / rs->a2)), two_inv_a2((T)(2.0 / rs->a2)), h3((T)(3.0 * rs->H)),
        pm2((T)(2.0 * rs->p_mean)) {}
};

// k components of mode m in T (FP64: the reference's expressions; FP32: the
// same products in single precision)
template <typename T> struct ModeK {
  T kx, ky, kz, ksq;
};
template <typename T>
__device__ __forceinline__ ModeK<T> mode_k(const Geom &g, Mode m) {
  ModeK<T> q;
  if constexpr (sizeof(T) == 8) {
    q.kx = kxf_of(g, m.i);
    q.ky = kyf_of(g, m.j);
    q.kz = kzf_of(g, m.k);
    q.ksq = ksq64(g, m.i, m.j, m.k);
  } else {
    q.kx = (float)g.kxu * (float)((m.i > g.nx / 2) ? (m.i - g.nx) : m.i);
    q.ky = (float)g.kyu * (float)((m.j > g.ny / 2) ? (m.j - g.ny) : m.j);
    q.kz = (float)g.kzu * (float)m.k;
    int ia = (m.i > g.nx / 2) ? (g.nx - m.i) : m.i;
    int ja = (m.j > g.ny / 2) ? (g.ny - m.j) : m.j;
    q.ksq = (float)g.kz2 * (float)m.k * (float)m.k;
    q.ksq += (float)g.kx2 * (float)ia * (float)ia;
    q.ksq += (float)g.ky2 * (float)ja * (float)ja;
  }
  return q;
}

// The two projected sources n0, n1 of mode m (id != 0) from the six S_ij
// spectra v (xx, xy, xz, yy, yz, zz), toolbox.c:363-397.
template <typename T>
__device__ __forceinline__ void tensor_sources(Mode m, const ModeK<T> &q, const C2<T> (&v)[6],
                                               C2<T> &n0, C2<T> &n1) {
  const T kx = q.kx, ky = q.ky, kz = q.kz;
  const T inv_ksq = (T)1.0 / q.ksq;
  const T fx = kx * inv_ksq, fy = ky * inv_ksq, fz = kz * inv_ksq;
  const C2<T> v0 = v[0], v1 = v[1], v2 = v[2], v3 = v[3], v4 = v[4], v5 = v[5];
#define CL(c, a, b) mk2c<T>(a.x c b.x, a.y c b.y)
#define SC(f, a) mk2c<T>((f) * a.x, (f) * a.y)
  C2<T> t1 = CL(+, CL(+, CL(+, SC(kx * fx, v0), SC(ky * fy, v3)), SC(kz * fz, v5)),
                SC((T)2.0, CL(+, CL(+, SC(kx * fy, v1), SC(kx * fz, v2)), SC(ky * fz, v4))));
  C2<T> t2 = CL(+, CL(+, v0, v3), v5);
  C2<T> S1 = CL(+, t1, t2), S2 = CL(-, t1, t2);
  // |kz| > DBL_EPSILON and |ky| > DBL_EPSILON of toolbox.c:377, 382: the
  // grid components are either exactly 0 or at least 2 pi / L
  if (m.k != 0) {
    C2<T> k1 = CL(+, CL(+, SC(kx, v0), SC(ky, v1)), SC(kz, v2));
    C2<T> k2 = CL(+, CL(+, SC(kx, v1), SC(ky, v3)), SC(kz, v4));
    n0 = CL(+, CL(-, v0, SC((T)2.0 * fx, k1)), SC((T)0.5, CL(+, SC(fx * kx, S1), S2)));
    n1 = CL(+, CL(-, CL(-, v1, SC(fx, k2)), SC(fy, k1)), SC((T)0.5 * fx * ky, S1));
  } else if (m.j != 0) {
    C2<T> k1 = CL(+, CL(+, SC(kx, v0), SC(ky, v1)), SC(kz, v2));
    C2<T> k3 = CL(+, CL(+, SC(kx, v2), SC(ky, v4)), SC(kz, v5));
    n0 = CL(+, CL(-, v0, SC((T)2.0 * fx, k1)), SC((T)0.5, CL(+, SC(fx * kx, S1), S2)));
    n1 = CL(+, CL(-, CL(-, v2, SC(fx, k3)), SC(fz, k1)), SC((T)0.5 * fx * kz, S1));
  } else {
    C2<T> k2 = CL(+, CL(+, SC(kx, v1), SC(ky, v3)), SC(kz, v4));
    C2<T> k3 = CL(+, CL(+, SC(kx, v2), SC(ky, v4)), SC(kz, v5));
    n0 = CL(+, CL(-, v3, SC((T)2.0 * fy, k2)), SC((T)0.5, CL(+, SC(fy * ky, S1), S2)));
    n1 = CL(+, CL(-, CL(-, v4, SC(fy, k3)), SC(fz, k2)), SC((T)0.5 * fy * kz, S1));
  }
#undef CL
#undef SC
}

// The same projection as coefficients: n0 = sum_a alpha_a v_a and
// n1 = sum_a beta_a v_a (the expressions above are linear in v), for one
// spectrum a at a time.  With T1 = (kx fx, 2 kx fy, 2 kx fz, ky fy, 2 ky fz,
// kz fz), T2 = (1, 0, 0, 1, 0, 1), S1 = T1 + T2, S2 = T1 - T2, K1 = (kx, ky,
// kz, 0, 0, 0), K2 = (0, kx, 0, ky, kz, 0), K3 = (0, 0, kx, 0, ky, kz):
//   kz index != 0:        alpha = e0 - 2 fx K1 + (fx kx S1 + S2) / 2,
//                         beta  = e1 - fx K2 - fy K1 + fx ky S1 / 2
//   kz = 0, ky index != 0: alpha as above, beta = e2 - fx K3 - fz K1 + fx kz S1 / 2
//   kz = ky = 0:           alpha = e3 - 2 fy K2 + (fy ky S1 + S2) / 2,
//                         beta  = e4 - fy K3 - fz K2 + fy kz S1 / 2
// (e_b the unit vector of spectrum b).  branch: 0, 1, 2 for the three cases.
template <typename T>
__device__ __forceinline__ void tensor_coef(int a, int branch, T kx, T ky, T kz, T fx, T fy, T fz,
                                            T &alpha, T &beta) {
  const T t1 = a == 0 ? kx * fx : a == 1 ? (T)2.0 * kx * fy : a == 2 ? (T)2.0 * kx * fz
             : a == 3 ? ky * fy : a == 4 ? (T)2.0 * ky * fz : kz * fz;
  const T t2 = (a == 0 || a == 3 || a == 5) ? (T)1.0 : (T)0.0;
  const T s1 = t1 + t2, s2 = t1 - t2;
  const T k1 = a == 0 ? kx : a == 1 ? ky : a == 2 ? kz : (T)0.0;
  const T k2 = a == 1 ? kx : a == 3 ? ky : a == 4 ? kz : (T)0.0;
  const T k3 = a == 2 ? kx : a == 4 ? ky : a == 5 ? kz : (T)0.0;
  if (branch < 2) {
    alpha = (a == 0 ? (T)1.0 : (T)0.0) - (T)2.0 * fx * k1 + (T)0.5 * (fx * kx * s1 + s2);
    if (branch == 0)
      beta = (a == 1 ? (T)1.0 : (T)0.0) - fx * k2 - fy * k1 + (T)0.5 * fx * ky * s1;
    else
      beta = (a == 2 ? (T)1.0 : (T)0.0) - fx * k3 - fz * k1 + (T)0.5 * fx * kz * s1;
  } else {
    alpha = (a == 3 ? (T)1.0 : (T)0.0) - (T)2.0 * fy * k2 + (T)0.5 * (fy * ky * s1 + s2);
    beta = (a == 4 ? (T)1.0 : (T)0.0) - fy * k3 - fz * k2 + (T)0.5 * fy * kz * s1;
  }
}

// coefficient j of a next-stage combination in T
template <typename T>
__device__ __forceinline__ T nl_coef(const NextLin &nl, int j) {
  if constexpr (sizeof(T) == 4) {
    return nl.coeff[j];
  } else {
    return nl.coef[j];
  }
}
template <typename T>
__device__ __forceinline__ T nl_self(const NextLin &nl) {
  if constexpr (sizeof(T) == 4) {
    return nl.selff;
  } else {
    return nl.self;
  }
}
// next-stage input at complex element e of the state (V = C2<T>): base +
// dt (sum_j coef_j k_j + self o), written to y
template <typename T>
__device__ __forceinline__ void nl_apply_c(const NextLin &nl, T dt, long long e, C2<T> o,
                                           C2<T> *y) {
  typedef C2<T> V;
  T ax = 0, ay = 0;
#pragma unroll
  for (int j = 0; j < kMaxTerms; ++j) {
    if (j < nl.n) {
      const V kv = reinterpret_cast<const V *>(nl.k[j])[e];
      const T cj = nl_coef<T>(nl, j);
      ax += cj * kv.x;
      ay += cj * kv.y;
    }
  }
  const T cs = nl_self<T>(nl);
  ax += cs * o.x;
  ay += cs * o.y;
  const V bv = reinterpret_cast<const V *>(nl.base)[e];
  y[e] = mk2c<T>(bv.x + dt * ax, bv.y + dt * ay);
}

// The equation of motion of mode id from its sources n0, n1 (zero for the
// zero mode) and k^2: h1' = dh1, h2' = dh2,
// dh1' = -(2 <p> + k^2/a^2) h1 - 3 H dh1 + 2/a^2 n0 (and dh2'), reading the
// tensor segments of y and writing those of out; NEXT: also the next stage's
// input at the same entries of y (nl, dt = the step size in T).  Returns the
// largest |component| of the two dh' values (the FP32 noise scale of the
// tensor sources, see k_dopri_final).
// the tensor entries of mode id: h1, h2, dh1, dh2 (complex values at 2 id of
// each segment; Nh1, Next are even)
template <typename T>
struct HVals {
  C2<T> h1, h2, d1, d2;
};
template <typename T>
__device__ __forceinline__ void tensor_load(const Geom &g, long long id, const T *y, HVals<T> &v) {
  const long long N = g.N, Next = g.Next;
  const long long Nh1 = 4 * N, Nh2 = Nh1 + Next, Ndh1 = Nh2 + Next, Ndh2 = Ndh1 + Next;
  const C2<T> *yv = reinterpret_cast<const C2<T> *>(y);
  v.h1 = yv[Nh1 / 2 + id];
  v.h2 = yv[Nh2 / 2 + id];
  v.d1 = yv[Ndh1 / 2 + id];
  v.d2 = yv[Ndh2 / 2 + id];
}

// h' = dh (unless skip_pos) and dh' of mode id into out; returns dh1', dh2'
template <typename T>
__device__ __forceinline__ void tensor_eom_core(const Geom &g, long long id, C2<T> n0, C2<T> n1,
                                                T ksq, const TensorConsts<T> &tc,
                                                const HVals<T> &v, T *__restrict__ out,
                                                int skip_pos, C2<T> &o3, C2<T> &o4) {
  const long long N = g.N, Next = g.Next;
  const long long Nh1 = 4 * N, Nh2 = Nh1 + Next, Ndh1 = Nh2 + Next, Ndh2 = Ndh1 + Next;
  const T tm = -(tc.pm2 + ksq * tc.inv_a2);
  C2<T> *ov = reinterpret_cast<C2<T> *>(out);
  o3 = mk2c<T>(tm * v.h1.x - tc.h3 * v.d1.x + tc.two_inv_a2 * n0.x,
               tm * v.h1.y - tc.h3 * v.d1.y + tc.two_inv_a2 * n0.y);
  o4 = mk2c<T>(tm * v.h2.x - tc.h3 * v.d2.x + tc.two_inv_a2 * n1.x,
               tm * v.h2.y - tc.h3 * v.d2.y + tc.two_inv_a2 * n1.y);
  if (!skip_pos) {
    ov[Nh1 / 2 + id] = v.d1;
    ov[Nh2 / 2 + id] = v.d2;
  }
  ov[Ndh1 / 2 + id] = o3;
  ov[Ndh2 / 2 + id] = o4;
}

template <typename T, bool NEXT>
__device__ __forceinline__ T tensor_eom(const Geom &g, long long id, C2<T> n0, C2<T> n1, T ksq,
                                           const TensorConsts<T> &tc, T *y, T *__restrict__ out,
                                           const NextLin &nl, T dt) {
  const long long N = g.N, Next = g.Next;
  const long long Nh1 = 4 * N, Nh2 = Nh1 + Next, Ndh1 = Nh2 + Next, Ndh2 = Ndh1 + Next;
  typedef C2<T> V;
  V *yv = reinterpret_cast<V *>(y);
  const long long e1 = Nh1 / 2 + id, e2 = Nh2 / 2 + id, e3 = Ndh1 / 2 + id, e4 = Ndh2 / 2 + id;
  HVals<T> hv;
  tensor_load<T>(g, id, y, hv);
  const V d1 = hv.d1, d2 = hv.d2;
  V o3, o4;
  tensor_eom_core<T>(g, id, n0, n1, ksq, tc, hv, out, nl.skip_pos, o3, o4);
  if constexpr (NEXT) {
    nl_apply_c<T>(nl, dt, e1, d1, yv);
    nl_apply_c<T>(nl, dt, e2, d2, yv);
    nl_apply_c<T>(nl, dt, e3, o3, yv);
    nl_apply_c<T>(nl, dt, e4, o4, yv);
  }
  return fmax(fmax(fabs(o3.x), fabs(o3.y)), fmax(fabs(o4.x), fabs(o4.y)));
}

// the largest dh' of a k vector into its homogeneous slot 7 (zeroed by the
// reduction-finish kernel of the same RHS): warp maximum, one atomic per warp
template <typename T>
__device__ __forceinline__ void dh_max_store(T mx, double *ksc) {
  double v = (double)mx;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0 && v > 0.0)
    atomicMax(reinterpret_cast<unsigned long long *>(ksc + 7),
              (unsigned long long)__double_as_longlong(v));
}

}  // namespace ih
