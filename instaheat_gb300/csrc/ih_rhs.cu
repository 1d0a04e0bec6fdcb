// ih_rhs.cu -- the right-hand side mk_rhs (src/toolbox.c:75-88) and its
// helpers on GB300: filter, pointwise equations of motion, tensor sources,
// reductions, diagnostics, initial conditions and the psi constraint solve.
//
// One RHS evaluation (GW on, filter and output off) is this launch sequence:
//   zr2c(phi) -> Z                                    z spectrum of phi
//   x round trip(Z): d/dx Z, d2/dx2 Z                 (derivatives along one
//   y round trip(Z): d/dy Z, laplacian                 axis commute with the
//                                                      other axes' transforms)
//   z fused: 4 c2r (d/dz from Z), grad^2, rho, p, FP64 block sums,
//            6 products, 6 r2c(z)
//   reduce_finish: <rho>, <p>, H, homogeneous RHS parts
//   y fwd, x fwd (6 arrays)                           S_ij hat
//   update_h: TT projection + h'' (toolbox.c:311-397)
//   update_phi_psi (toolbox.c:282-299)
// With the filter or output flag phihat itself is formed (zr2c, y, x), then
// the fused inverse x pass (i k_a phihat / N, -k^2 phihat / N) and a 4-array
// inverse y pass feed the same z pass.  Either way the reference's 7 r2c +
// 4 c2r with the spectral multiplies, the pointwise products and the
// reductions folded into the FFT passes.
#include <float.h>
#include <math.h>
#include "ih_internal.cuh"
#include "ih_tensor.cuh"
#include "ih_fftcore.cuh"

namespace ih {

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_min(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
// block reductions; all threads must call; result valid in thread 0
__device__ double block_sum(double v) {
  __shared__ double sh[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)((blockDim.x + 31) / 32); ++i) r += sh[i];
  return r;
}
__device__ double block_max(double v) {
  __shared__ double sh[32];
  v = warp_max(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = -INFINITY;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)((blockDim.x + 31) / 32); ++i) r = fmax(r, sh[i]);
  return r;
}
__device__ double block_min(double v) {
  __shared__ double sh[32];
  v = warp_min(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = INFINITY;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)((blockDim.x + 31) / 32); ++i) r = fmin(r, sh[i]);
  return r;
}


// ---------------------------------------------------------------------------
// filter mask (setup.c:710-754), kept in T
template <typename T>
__global__ void k_mask_init(T *mask, Geom g) {
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < g.M;
       id += (long long)gridDim.x * blockDim.x) {
    Mode m = mode_of(id, g);
    double frac = fabs(kxf_of(g, m.i)) / g.kxmax;
    frac = fmax(frac, fabs(kyf_of(g, m.j)) / g.kymax);
    frac = fmax(frac, fabs(kzf_of(g, m.k)) / g.kzmax);
    mask[id] = (T)exp(-36.0 * pow(frac, 36.0));
  }
}

// capply_filter for the four real fields at once (toolbox.c:160-171,
// 596-626): spec[4] = phihat * mask (kept for the derivatives), spec[0] =
// phihat * mask / N, spec[1..3] = {dphi, psi, dpsi}hat * mask / N; when
// keep_psi, spec[5] = psihat * mask.  Mixed form: the k = 0 value / N of each
// fluctuation field moves into the FP64 scalar and is zeroed in the spectrum.
template <typename T, bool MIXED>
__global__ void k_filter_spectra(C2<T> *spec, const T *mask, long long M,
                                 double invN, int keep_psi, double *ysc) {
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < M;
       id += (long long)gridDim.x * blockDim.x) {
    const T mk = mask[id];
    const T s = (T)invN;
    C2<T> ph = spec[4 * M + id];
    ph.x *= mk;
    ph.y *= mk;
    C2<T> d0 = mk2c<T>(ph.x * s, ph.y * s);
    C2<T> v1 = spec[M + id], v2 = spec[2 * M + id], v3 = spec[3 * M + id];
    v1.x *= mk; v1.y *= mk;
    v2.x *= mk; v2.y *= mk;
    v3.x *= mk; v3.y *= mk;
    if (keep_psi) spec[5 * M + id] = v2;
    v1.x *= s; v1.y *= s;
    v2.x *= s; v2.y *= s;
    v3.x *= s; v3.y *= s;
    if (MIXED && id == 0) {
      ysc[0] += (double)d0.x;
      ysc[1] += (double)v1.x;
      ysc[2] += (double)v2.x;
      ysc[3] += (double)v3.x;
      d0 = mk2c<T>(0, 0);
      v1 = d0;
      v2 = d0;
      v3 = d0;
    }
    spec[4 * M + id] = ph;
    spec[id] = d0;
    spec[M + id] = v1;
    spec[2 * M + id] = v2;
    spec[3 * M + id] = v3;
  }
}

// <rho>, <p>, H and the homogeneous parts of the RHS (one block).
// toolbox.c:241-242 (means), 286-287 (H), 87 (da/dt).
__global__ void k_reduce_finish(const double *partials, int nblk, Geom g,
                                const double *ysc, double *ksc, RhsScalars *rs,
                                int mixed) {
  double sr = 0.0, sp = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    sr += partials[2 * b];
    sp += partials[2 * b + 1];
  }
  sr = block_sum(sr);
  __syncthreads();
  sp = block_sum(sp);
  if (threadIdx.x != 0) return;
  const double m2 = g.mass * g.mass;
  const double phib = ysc[0], pib = ysc[1], psib = ysc[2], dpsib = ysc[3], a = ysc[4];
  double rho_bar = 0.0, p_bar = 0.0;
  if (mixed) {
    double kin = (0.5 - psib) * pib * pib, pot = 0.5 * m2 * phib * phib;
    rho_bar = kin + pot;
    p_bar = kin - pot;
  }
  const double rho_mean = rho_bar + sr / (double)g.N;
  const double p_mean = p_bar + sp / (double)g.N;
  const double H = sqrt(rho_mean / 3.0);
  RhsScalars r;
  r.rho_mean = rho_mean;
  r.p_mean = p_mean;
  r.H = H;
  r.a = a;
  r.a2 = a * a;
  r.rho_bar = rho_bar;
  r.p_bar = p_bar;
  r.dphi_mean = 0.0;
  r.phi_mean = 0.0;
  r.ddphi_mean = 0.0;
  r.nonfinite = !(isfinite(rho_mean) && isfinite(p_mean));
  r.pad = 0;
  *rs = r;
  if (mixed) {
    ksc[0] = pib;
    ksc[1] = -(3.0 * H - 4.0 * dpsib) * pib - (1.0 + 2.0 * psib) * m2 * phib;
    ksc[2] = dpsib;
    ksc[3] = 0.5 * p_bar + (psib - 0.5) * p_mean - 4.0 * H * dpsib;
  } else {
    ksc[0] = ksc[1] = ksc[2] = ksc[3] = 0.0;
  }
  ksc[4] = a * H;
  ksc[5] = ksc[6] = ksc[7] = 0.0;
}

// update_phi_psi (toolbox.c:282-299); mixed form: fluctuation parts only,
// the homogeneous parts were written by k_reduce_finish.  W points per
// thread (one 16-byte vector per array).  NEXT: also the next stage's input
// (nl) at the four real segments, written over y -- each element of y is
// read, then overwritten, by the same thread.
template <typename T> struct VecW;
template <> struct VecW<float> {
  using V = float4;
  static constexpr int W = 4;
};
template <> struct VecW<double> {
  using V = double2;
  static constexpr int W = 2;
};
template <typename T>
__device__ __forceinline__ void ld_w(const T *p, T (&v)[VecW<T>::W]) {
  if constexpr (sizeof(T) == 4) {
    const float4 q = *reinterpret_cast<const float4 *>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  } else {
    const double2 q = *reinterpret_cast<const double2 *>(p);
    v[0] = q.x; v[1] = q.y;
  }
}
template <typename T>
__device__ __forceinline__ void st_w(T *p, const T (&v)[VecW<T>::W]) {
  if constexpr (sizeof(T) == 4) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
  }
}

template <typename T, bool MIXED, bool NEXT>
__global__ void k_update_phi_psi(T *y, const double *ysc, const T *__restrict__ lap,
                                 const T *__restrict__ p, T *__restrict__ out,
                                 const RhsScalars *rs, long long N, double mass,
                                 const NextLin nl) {
  constexpr int W = VecW<T>::W;
  const double a2d = rs->a2, Hd = rs->H, pmd = rs->p_mean;
  const T inv_a2 = (T)(1.0 / a2d), H = (T)Hd, h3 = (T)(3.0 * Hd), pm = (T)pmd;
  const T m2 = (T)(mass * mass);
  T phib = 0, pib = 0, psib = 0, dpsib = 0;
  if (MIXED) {
    phib = (T)ysc[0];
    pib = (T)ysc[1];
    psib = (T)ysc[2];
    dpsib = (T)ysc[3];
  }
  const T dt = NEXT ? (T)*nl.dt : (T)0;
  const long long nv = N / W;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    const long long i0 = v * W;
    T ph[W], dph[W], ps[W], dps[W], l[W], pp[W], o1[W], o3[W];
    ld_w<T>(y + i0, ph);
    ld_w<T>(y + N + i0, dph);
    ld_w<T>(y + 2 * N + i0, ps);
    ld_w<T>(y + 3 * N + i0, dps);
    ld_w<T>(lap + i0, l);
    ld_w<T>(p + i0, pp);
#pragma unroll
    for (int w = 0; w < W; ++w) {
      if (!MIXED) {
        o1[w] = ((T)1.0 + (T)4.0 * ps[w]) * l[w] * inv_a2 - (h3 - (T)4.0 * dps[w]) * dph[w] -
                ((T)1.0 + (T)2.0 * ps[w]) * (m2 * ph[w]);
        o3[w] = (T)0.5 * pp[w] + (ps[w] - (T)0.5) * pm - (T)4.0 * H * dps[w];
      } else {
        T psf = psib + ps[w], dpsf = dpsib + dps[w];
        o1[w] = ((T)1.0 + (T)4.0 * psf) * l[w] * inv_a2 + (T)4.0 * dps[w] * pib -
                (h3 - (T)4.0 * dpsf) * dph[w] - (T)2.0 * ps[w] * m2 * phib -
                ((T)1.0 + (T)2.0 * psf) * m2 * ph[w];
        o3[w] = (T)0.5 * pp[w] + ps[w] * pm - (T)4.0 * H * dps[w];
      }
    }
    if (!nl.skip_pos) {
      st_w<T>(out + i0, dph);
      st_w<T>(out + 2 * N + i0, dps);
    }
    st_w<T>(out + N + i0, o1);
    st_w<T>(out + 3 * N + i0, o3);
    if constexpr (NEXT) {
#pragma unroll
      for (int seg = 0; seg < 4; ++seg) {
        const T *o = seg == 0 ? dph : seg == 1 ? o1 : seg == 2 ? dps : o3;
        const long long e = seg * N + i0;
        T acc[W], x[W];
#pragma unroll
        for (int w = 0; w < W; ++w) acc[w] = 0;
#pragma unroll
        for (int j = 0; j < kMaxTerms; ++j) {
          if (j < nl.n) {
            ld_w<T>(reinterpret_cast<const T *>(nl.k[j]) + e, x);
            const T cj = nl_coef<T>(nl, j);
#pragma unroll
            for (int w = 0; w < W; ++w) acc[w] += cj * x[w];
          }
        }
        const T cs = nl_self<T>(nl);
#pragma unroll
        for (int w = 0; w < W; ++w) acc[w] += cs * o[w];
        ld_w<T>(reinterpret_cast<const T *>(nl.base) + e, x);
#pragma unroll
        for (int w = 0; w < W; ++w) x[w] = x[w] + dt * acc[w];
        st_w<T>(y + e, x);
      }
    }
  }
}

// the homogeneous parts of the next stage input (after every kernel that
// reads those of the current one): outsc = basesc + dt (sum_j coef_j ksc_j +
// self ksc), in the order of the stand-alone combination
__global__ void k_next_sc(const NextLin nl, const double *ksc, double *outsc) {
  const int s = threadIdx.x;
  if (s >= 5) return;
  const double dt = *nl.dt;
  double acc = 0.0;
  for (int j = 0; j < nl.n; ++j) acc += nl.coef[j] * nl.ksc[j][s];
  acc += nl.self * ksc[s];
  outsc[s] = nl.basesc[s] + dt * acc;
}

// update_h with the TT projection (toolbox.c:311-346, 363-397).  s holds the
// six S_ij spectra, spectra 4 and 5 at s + 5M.
// NEXT: also the next stage's input at the tensor entries of y (nl).
template <typename T, bool NEXT>
__global__ void __launch_bounds__(256, (sizeof(T) == 4 ? (NEXT ? 3 : 4) : 2)) k_update_h(
    const C2<T> *__restrict__ s, T *y, T *__restrict__ out, const RhsScalars *rs, Geom g,
    const NextLin nl, double *outsc) {
  const long long M = g.M;
  const TensorConsts<T> tc(rs);
  const T dt = NEXT ? (T)*nl.dt : (T)0;
  T mx = 0;
  const unsigned mz_magic = g.mz_magic;
  const int mz_shift = g.mz_shift, logny = g.logny;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < M;
       id += (long long)gridDim.x * blockDim.x) {
    // mode (i, j, k) of the half spectrum: one division by mz via a
    // multiply-high (32-bit ids: M < 2^31)
    const unsigned uid = (unsigned)id;
    const unsigned r = (__umulhi(uid, mz_magic) + uid) >> mz_shift;
    Mode m;
    m.k = (int)(uid - r * (unsigned)g.mz);
    if (g.pow2) {
      m.j = (int)(r & (unsigned)(g.ny - 1));
      m.i = (int)(r >> logny);
    } else {
      m.j = (int)(r % (unsigned)g.ny);
      m.i = (int)(r / (unsigned)g.ny);
    }
    C2<T> n0 = mk2c<T>(0, 0), n1 = mk2c<T>(0, 0);
    T ksq = 0;
    if (id != 0) {  // the zero mode has no sources (its spectra are not read)
      const C2<T> v[6] = {s[id], s[M + id], s[2 * M + id], s[3 * M + id], s[5 * M + id],
                          s[6 * M + id]};
      const ModeK<T> q = mode_k<T>(g, m);
      ksq = q.ksq;
      tensor_sources<T>(m, q, v, n0, n1);
    }
    mx = fmax(mx, tensor_eom<T, NEXT>(g, id, n0, n1, ksq, tc, y, out, nl, dt));
  }
  dh_max_store<T>(mx, outsc);
}

// update_h without the next stage input, one mode ahead: the ten loads of
// the next mode (six S_ij, h1, h2, dh1, dh2) are issued before the
// projection arithmetic of the current one, so a warp keeps them in flight
// through its arithmetic
template <typename T>
__global__ void __launch_bounds__(256, 3) k_update_h_pf(
    const C2<T> *__restrict__ s, const T *__restrict__ y, T *__restrict__ out,
    const RhsScalars *rs, Geom g, int skip_pos, double *outsc) {
  const long long M = g.M;
  const TensorConsts<T> tc(rs);
  T mx = 0;
  const unsigned mz_magic = g.mz_magic;
  const int mz_shift = g.mz_shift, logny = g.logny;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  C2<T> v[6];
  HVals<T> hv;
  auto load = [&](long long q, C2<T>(&vv)[6], HVals<T> &h) {
    if (q != 0) {  // the zero mode has no sources (its spectra are not read)
      vv[0] = s[q];
      vv[1] = s[M + q];
      vv[2] = s[2 * M + q];
      vv[3] = s[3 * M + q];
      vv[4] = s[5 * M + q];
      vv[5] = s[6 * M + q];
    } else {
#pragma unroll
      for (int a = 0; a < 6; ++a) vv[a] = mk2c<T>(0, 0);
    }
    tensor_load<T>(g, q, y, h);
  };
  if (id < M) load(id, v, hv);
  while (id < M) {
    const long long nid = id + stride;
    C2<T> vn[6];
    HVals<T> hn;
    if (nid < M) {
      load(nid, vn, hn);
    } else {
#pragma unroll
      for (int a = 0; a < 6; ++a) vn[a] = mk2c<T>(0, 0);
      hn.h1 = hn.h2 = hn.d1 = hn.d2 = mk2c<T>(0, 0);
    }
    const unsigned uid = (unsigned)id;
    const unsigned r = (__umulhi(uid, mz_magic) + uid) >> mz_shift;
    Mode m;
    m.k = (int)(uid - r * (unsigned)g.mz);
    if (g.pow2) {
      m.j = (int)(r & (unsigned)(g.ny - 1));
      m.i = (int)(r >> logny);
    } else {
      m.j = (int)(r % (unsigned)g.ny);
      m.i = (int)(r / (unsigned)g.ny);
    }
    C2<T> n0 = mk2c<T>(0, 0), n1 = mk2c<T>(0, 0);
    T ksq = 0;
    if (id != 0) {
      const ModeK<T> q = mode_k<T>(g, m);
      ksq = q.ksq;
      tensor_sources<T>(m, q, v, n0, n1);
    }
    C2<T> o3, o4;
    tensor_eom_core<T>(g, id, n0, n1, ksq, tc, hv, out, skip_pos, o3, o4);
    mx = fmax(mx, fmax(fmax(fabs(o3.x), fabs(o3.y)), fmax(fabs(o4.x), fabs(o4.y))));
#pragma unroll
    for (int a = 0; a < 6; ++a) v[a] = vn[a];
    hv = hn;
    id = nid;
  }
  dh_max_store<T>(mx, outsc);
}

// The last forward x pass of the six S_ij spectra (arrays 0..3, 5, 6 of
// spec; z and y passes done) and update_h, writing the tensor segments of
// out: x passes then k_update_h, or the fused k_fft_x_tensor, as the
// autotuner chose (Ctx::tensor_fused).  next: the tensor entries of the next
// stage input too (in y).
template <typename T>
static int tensor_last_pass_t(Ctx *c, C2<T> *s, T *y, T *out, double *outsc,
                              const NextLin *next, bool x_done) {
  const Geom &g = c->g;
  const long long M = g.M;
  if (!x_done) {
    if (c->tensor_fused && g.pow2) return fft_x_tensor<T>(c, s, s + 5 * M, y, out, outsc, next);
    IH_TRY((fft_xy<T>(c, s, M, 4, 0, -1)));
    IH_TRY((fft_xy<T>(c, s + 5 * M, M, 2, 0, -1)));
  }
  const unsigned gm = grid_for(M, 256, 4);
  prof_begin(c, KK_UPDATE_H);
  if (next) {
    k_update_h<T, true><<<gm, 256, 0, c->stream>>>(s, y, out, c->rs, g, *next, outsc);
  } else if constexpr (sizeof(T) == 4) {
    k_update_h_pf<T><<<gm, 256, 0, c->stream>>>(s, y, out, c->rs, g, c->skip_pos, outsc);
  } else {  // FP64: ALU-bound; the prefetching form would spill
    NextLin none{};
    none.skip_pos = c->skip_pos;
    k_update_h<T, false><<<gm, 256, 0, c->stream>>>(s, y, out, c->rs, g, none, outsc);
  }
  prof_end(c, KK_UPDATE_H,
           6.0 * M * sizeof(C2<T>) +
               ((c->skip_pos ? 6.0 : 8.0) + (next ? 4.0 * (next->n + 2) : 0.0)) * g.Next * sizeof(T));
  return check_launch(c, "k_update_h");
}
int tensor_last_pass(Ctx *c, void *spec, void *y, void *out, double *outsc,
                     const NextLin *next, bool x_done) {
  if (c->mixed)
    return tensor_last_pass_t<float>(c, (C2<float> *)spec, (float *)y, (float *)out, outsc, next,
                                     x_done);
  return tensor_last_pass_t<double>(c, (C2<double> *)spec, (double *)y, (double *)out, outsc,
                                    next, x_done);
}

// ---------------------------------------------------------------------------
// generic FP64 reductions of T arrays (deterministic two-stage)
template <typename T>
__global__ void k_partial_sum(const T *a, long long n, double *partials) {
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    s += (double)a[i];
  s = block_sum(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}
__global__ void k_finish_sum(const double *partials, int nb, double scale, double add,
                             double *out) {
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partials[b];
  s = block_sum(s);
  if (threadIdx.x == 0) *out = add + s * scale;
}

static int nblk_reduce(long long n) {
  long long b = (n + 1023) / 1024;
  if (b > 1024) b = 1024;
  if (b < 1) b = 1;
  return (int)b;
}

template <typename T>
static int mean_into(Ctx *c, const T *a, long long n, double *dev_out) {
  const int nb = nblk_reduce(n);
  k_partial_sum<T><<<nb, 256, 0, c->stream>>>(a, n, c->partials);
  IH_TRY(check_launch(c, "k_partial_sum"));
  k_finish_sum<<<1, 256, 0, c->stream>>>(c->partials, nb, 1.0 / (double)n, 0.0, dev_out);
  return check_launch(c, "k_finish_sum");
}

__global__ void k_add_scalar(double *dst, const double *src) { *dst += *src; }

// sum and sum of squares per block -> rms about the mean (FP64)
template <typename T>
__global__ void k_partial_sum2(const T *a, long long n, double *partials) {
  double s = 0.0, q = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = (double)a[i];
    s += v;
    q += v * v;
  }
  s = block_sum(s);
  __syncthreads();
  q = block_sum(q);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = s;
    partials[2 * blockIdx.x + 1] = q;
  }
}
__global__ void k_finish_rms(const double *partials, int nb, long long n, double *out) {
  double s = 0.0, q = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    s += partials[2 * b];
    q += partials[2 * b + 1];
  }
  s = block_sum(s);
  __syncthreads();
  q = block_sum(q);
  if (threadIdx.x == 0) {
    const double m = s / (double)n;
    *out = sqrt(fmax(q / (double)n - m * m, 0.0));
  }
}

int field_rms(Ctx *c, const void *arr, long long n, double *dev_out) {
  const int nb = nblk_reduce(n);
  if (c->mixed)
    k_partial_sum2<float><<<nb, 256, 0, c->stream>>>((const float *)arr, n, c->partials);
  else
    k_partial_sum2<double><<<nb, 256, 0, c->stream>>>((const double *)arr, n, c->partials);
  IH_TRY(check_launch(c, "k_partial_sum2"));
  k_finish_rms<<<1, 256, 0, c->stream>>>(c->partials, nb, n, dev_out);
  return check_launch(c, "k_finish_rms");
}

int reduce_mean_f64(Ctx *c, const double *arr, long long n, double *dev_out) {
  return mean_into<double>(c, arr, n, dev_out);
}

int reduce_mean(Ctx *c, const void *arr, long long n, double *dev_out) {
  if (c->mixed) return mean_into<float>(c, (const float *)arr, n, dev_out);
  return mean_into<double>(c, (const double *)arr, n, dev_out);
}

// ---------------------------------------------------------------------------
// conversions between the reference layout (FP64, Ntot) and a Vec
template <typename T>
__global__ void k_from_ref(const double *ref, T *fl, const double *means, long long N,
                           long long Nf) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < Nf;
       i += (long long)gridDim.x * blockDim.x) {
    double v = ref[i];
    if (means && i < 4 * N) v -= means[i / N];
    fl[i] = (T)v;
  }
}
template <typename T>
__global__ void k_to_ref(const T *fl, const double *sc, double *ref, long long N,
                         long long Nf) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < Nf;
       i += (long long)gridDim.x * blockDim.x) {
    double v = (double)fl[i];
    if (i < 4 * N) v += sc[i / N];
    ref[i] = v;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) ref[Nf] = sc[4];
}
__global__ void k_sc_from_ref(const double *ref, double *sc, const double *means,
                              long long Nf) {
  for (int s = 0; s < 4; ++s) sc[s] = means ? means[s] : 0.0;
  sc[4] = ref[Nf];
  sc[5] = sc[6] = sc[7] = 0.0;
}

int vec_from_ref(Ctx *c, const double *ref_dev, Vec &v) {
  const Geom &g = c->g;
  double *means = nullptr;
  if (c->mixed) {
    // FP64 segment means become the homogeneous parts
    means = c->diag + 4 * g.bins + 64;  // scratch slots
    for (int s = 0; s < 4; ++s) {
      const int nb = nblk_reduce(g.N);
      k_partial_sum<double><<<nb, 256, 0, c->stream>>>(ref_dev + s * g.N, g.N, c->partials);
      IH_TRY(check_launch(c, "k_partial_sum"));
      k_finish_sum<<<1, 256, 0, c->stream>>>(c->partials, nb, 1.0 / (double)g.N, 0.0, means + s);
      IH_TRY(check_launch(c, "k_finish_sum"));
    }
  }
  const unsigned gb = grid_for(g.Nf, 256, 4);
  if (c->mixed)
    k_from_ref<float><<<gb, 256, 0, c->stream>>>(ref_dev, (float *)v.fl, means, g.N, g.Nf);
  else
    k_from_ref<double><<<gb, 256, 0, c->stream>>>(ref_dev, (double *)v.fl, nullptr, g.N, g.Nf);
  IH_TRY(check_launch(c, "k_from_ref"));
  k_sc_from_ref<<<1, 1, 0, c->stream>>>(ref_dev, v.sc, means, g.Nf);
  return check_launch(c, "k_sc_from_ref");
}

int vec_to_ref(Ctx *c, const Vec &v, double *ref_dev) {
  const Geom &g = c->g;
  const unsigned gb = grid_for(g.Nf, 256, 4);
  if (c->mixed)
    k_to_ref<float><<<gb, 256, 0, c->stream>>>((const float *)v.fl, v.sc, ref_dev, g.N, g.Nf);
  else
    k_to_ref<double><<<gb, 256, 0, c->stream>>>((const double *)v.fl, v.sc, ref_dev, g.N, g.Nf);
  return check_launch(c, "k_to_ref");
}

int vec_copy(Ctx *c, const Vec &src, Vec &dst) {
  IH_CUDA(c, cudaMemcpyAsync(dst.fl, src.fl, c->tsize * c->g.Nf, cudaMemcpyDeviceToDevice,
                             c->stream));
  IH_CUDA(c, cudaMemcpyAsync(dst.sc, src.sc, sizeof(double) * kSc, cudaMemcpyDeviceToDevice,
                             c->stream));
  return IH_OK;
}

// ---------------------------------------------------------------------------
// diagnostics (toolbox.c:251-270, 435-484, 524-551, 567-582, 634-690)
template <typename T>
__global__ void k_power_spectrum(const C2<T> *c, Geom g, double *out) {
  extern __shared__ double hist[];
  for (int b = threadIdx.x; b < g.bins; b += blockDim.x) hist[b] = 0.0;
  __syncthreads();
  for (long long id = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; id < g.M;
       id += (long long)gridDim.x * blockDim.x) {
    Mode m = mode_of(id, g);
    C2<T> v = c[id];
    double p2 = (double)v.x * (double)v.x + (double)v.y * (double)v.y;
    if (fabs(kz_deriv(g, m.k)) > DBL_EPSILON) p2 *= 2.0;
    int idx = (int)trunc(g.bins * sqrt(ksq64(g, m.i, m.j, m.k)) / g.kmax - 1.0e-14);
    idx = min(max(idx, 0), g.bins - 1);
    atomicAdd(&hist[idx], p2 / (double)g.N);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < g.bins; b += blockDim.x) atomicAdd(&out[b], hist[b]);
}

template <typename T>
__global__ void k_gw_spectrum(const T *y, const RhsScalars *rs, Geom g, double rat,
                              double *out) {
  extern __shared__ double hist[];
  for (int b = threadIdx.x; b < g.bins; b += blockDim.x) hist[b] = 0.0;
  __syncthreads();
  const long long N = g.N, Next = g.Next;
  const long long Ndh1 = 4 * N + 2 * Next, Ndh2 = Ndh1 + Next;
  const double H = rs->H;
  const double fac = kPi * rat / (3.0 * H * H * g.lx * g.ly * g.lz);
  for (long long id = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; id < g.M;
       id += (long long)gridDim.x * blockDim.x) {
    Mode m = mode_of(id, g);
    double kx = kxf_of(g, m.i), ky = kyf_of(g, m.j), kz = kzf_of(g, m.k);
    double kx2 = kx * kx, ky2 = ky * ky, kz2 = kz * kz;
    double k2 = ksq64(g, m.i, m.j, m.k), k = sqrt(k2);
    double d1r = y[Ndh1 + 2 * id], d2r = y[Ndh2 + 2 * id];
    double d1i = y[Ndh1 + 2 * id + 1], d2i = y[Ndh2 + 2 * id + 1];
    double pw;
    if (fabs(kz) > DBL_EPSILON) {
      pw = 2.0 * k2 / (kz2 * (ky2 + kz2)) *
           ((kx2 + kz2) * (d1r * d1r + d1i * d1i) + 2.0 * kx * ky * (d1r * d2r + d1i * d2i) +
            (ky2 + kz2) * (d2r * d2r + d2i * d2i));
    } else if (fabs(ky) > DBL_EPSILON) {
      pw = 2.0 * (kx2 + ky2) / (ky2 * ky2) *
           ((kx2 + ky2) * (d1r * d1r + d1i * d1i) + ky2 * (d2r * d2r + d2i * d2i));
    } else {
      pw = 2.0 * (d1r * d1r + d1i * d1i + d2r * d2r + d2i * d2i);
    }
    if (fabs(kz_deriv(g, m.k)) > DBL_EPSILON) pw *= 2.0;
    int idx = (int)trunc(g.bins * k / g.kmax - 1.0e-14);
    idx = min(max(idx, 0), g.bins - 1);
    atomicAdd(&hist[idx], fac * k2 * k * pw / (double)N);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < g.bins; b += blockDim.x) atomicAdd(&out[b], hist[b]);
}

// -k^2 psihat / N (toolbox.c:177-184) into a work spectrum
template <typename T>
__global__ void k_lap_spectrum(const C2<T> *in, C2<T> *out, Geom g) {
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < g.M;
       id += (long long)gridDim.x * blockDim.x) {
    Mode m = mode_of(id, g);
    const double q = ksq64(g, m.i, m.j, m.k);
    C2<T> v = in[id];
    out[id] = mk2c<T>((T)(-(double)v.x * q / (double)g.N), (T)(-(double)v.y * q / (double)g.N));
  }
}

// per-block sums for the constraints: [sum ham^2, max |ham|, sum mom^2, max |mom|]
template <typename T>
__global__ void k_constraints(const T *y, const double *ysc, const T *lappsi, const T *rho,
                              const RhsScalars *rs, const double *means, long long N,
                              double *partials) {
  const double a2 = rs->a2, H = rs->H, h3 = 3.0 * H, rho_mean = rs->rho_mean;
  const double rho_off = rs->rho_bar - rho_mean;  // rho_i - <rho> = drho + rho_bar - <rho>
  const double phi_mean = means[0], dphi_mean = means[1];
  double hl2 = 0.0, hmax = 0.0, ml2 = 0.0, mmax = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    double ps = ysc[2] + (double)y[2 * N + i], dps = ysc[3] + (double)y[3 * N + i];
    double ph = ysc[0] + (double)y[i];
    double t1 = H * ps + dps;
    double ham = (double)lappsi[i] / a2 - h3 * t1 - 0.5 * ((double)rho[i] + rho_off);
    double mom = t1 - 0.5 * dphi_mean * (ph - phi_mean);
    hl2 += ham * ham;
    ml2 += mom * mom;
    hmax = fmax(hmax, fabs(ham));
    mmax = fmax(mmax, fabs(mom));
  }
  hl2 = block_sum(hl2);
  __syncthreads();
  ml2 = block_sum(ml2);
  __syncthreads();
  hmax = block_max(hmax);
  __syncthreads();
  mmax = block_max(mmax);
  if (threadIdx.x == 0) {
    partials[4 * blockIdx.x] = hl2;
    partials[4 * blockIdx.x + 1] = hmax;
    partials[4 * blockIdx.x + 2] = ml2;
    partials[4 * blockIdx.x + 3] = mmax;
  }
}
__global__ void k_constraints_finish(const double *partials, int nb, long long N,
                                     double *out) {
  double a = 0, b = 0, cc = 0, d = 0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    a += partials[4 * i];
    b = fmax(b, partials[4 * i + 1]);
    cc += partials[4 * i + 2];
    d = fmax(d, partials[4 * i + 3]);
  }
  a = block_sum(a);
  __syncthreads();
  b = block_max(b);
  __syncthreads();
  cc = block_sum(cc);
  __syncthreads();
  d = block_max(d);
  if (threadIdx.x == 0) {
    out[0] = a / (double)N;
    out[1] = b;
    out[2] = cc / (double)N;
    out[3] = d;
  }
}

// summary of a field x_i = add + a[i] (mean, corrected variance, min, max;
// toolbox.c:676-690, 744-754).  Two passes.
template <typename T>
__global__ void k_smry1(const T *a, double add, long long n, double *partials) {
  double s = 0.0, mn = INFINITY, mx = -INFINITY;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double v = add + (double)a[i];
    s += v;
    mn = fmin(mn, v);
    mx = fmax(mx, v);
  }
  s = block_sum(s);
  __syncthreads();
  mn = block_min(mn);
  __syncthreads();
  mx = block_max(mx);
  if (threadIdx.x == 0) {
    partials[3 * blockIdx.x] = s;
    partials[3 * blockIdx.x + 1] = mn;
    partials[3 * blockIdx.x + 2] = mx;
  }
}
__global__ void k_smry1_finish(const double *partials, int nb, long long n, double *out) {
  double s = 0, mn = INFINITY, mx = -INFINITY;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    s += partials[3 * i];
    mn = fmin(mn, partials[3 * i + 1]);
    mx = fmax(mx, partials[3 * i + 2]);
  }
  s = block_sum(s);
  __syncthreads();
  mn = block_min(mn);
  __syncthreads();
  mx = block_max(mx);
  if (threadIdx.x == 0) {
    out[0] = s / (double)n;
    out[2] = mn;
    out[3] = mx;
  }
}
template <typename T>
__global__ void k_smry2(const T *a, double add, long long n, const double *meanp,
                        double *partials) {
  const double mean = *meanp;
  double s1 = 0.0, s2 = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double d = add + (double)a[i] - mean;
    s1 += d * d;
    s2 += d;
  }
  s1 = block_sum(s1);
  __syncthreads();
  s2 = block_sum(s2);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = s1;
    partials[2 * blockIdx.x + 1] = s2;
  }
}
__global__ void k_smry2_finish(const double *partials, int nb, long long n, double *out) {
  double s1 = 0, s2 = 0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    s1 += partials[2 * i];
    s2 += partials[2 * i + 1];
  }
  s1 = block_sum(s1);
  __syncthreads();
  s2 = block_sum(s2);
  if (threadIdx.x == 0) out[1] = (s1 - s2 * s2 / (double)n) / (double)(n - 1);
}

// homogeneous add for a per-point field whose FP64 part lives in a scalar
__global__ void k_copy_scalar(const double *src, double *dst) { *dst = *src; }

template <typename T>
static int summary(Ctx *c, const T *a, const double *add_dev_unused, double add, long long n,
                   double *out) {
  (void)add_dev_unused;
  const int nb = nblk_reduce(n);
  k_smry1<T><<<nb, 256, 0, c->stream>>>(a, add, n, c->partials);
  IH_TRY(check_launch(c, "k_smry1"));
  k_smry1_finish<<<1, 256, 0, c->stream>>>(c->partials, nb, n, out);
  IH_TRY(check_launch(c, "k_smry1_finish"));
  k_smry2<T><<<nb, 256, 0, c->stream>>>(a, add, n, out, c->partials);
  IH_TRY(check_launch(c, "k_smry2"));
  k_smry2_finish<<<1, 256, 0, c->stream>>>(c->partials, nb, n, out);
  return check_launch(c, "k_smry2_finish");
}

__global__ void k_set_scalar(double *dst, double v) { *dst = v; }

int variance_f64(Ctx *c, const double *arr, long long n, double mean, double *dev_out) {
  k_set_scalar<<<1, 1, 0, c->stream>>>(dev_out, mean);
  IH_TRY(check_launch(c, "k_set_scalar"));
  const int nb = nblk_reduce(n);
  k_smry2<double><<<nb, 256, 0, c->stream>>>(arr, 0.0, n, dev_out, c->partials);
  IH_TRY(check_launch(c, "k_smry2"));
  k_smry2_finish<<<1, 256, 0, c->stream>>>(c->partials, nb, n, dev_out);
  return check_launch(c, "k_smry2_finish");
}

// The output flag (toolbox.c:251-270), in two parts around the fused z pass
// (which reuses spec[0..3], spec[5], spec[6] for the GW products).
// output_pre: psi power spectrum and the laplacian of psi (toolbox.c:172-184)
// from spec[5] = psihat (filtered when the filter ran).
template <typename T>
static int output_pre(Ctx *c, const Vec &y, int psi_ready) {
  const Geom &g = c->g;
  const long long M = g.M, N = g.N;
  C2<T> *spec = (C2<T> *)c->spec[0];
  const T *yfl = (const T *)y.fl;
  double *d = c->diag;
  const int bins = g.bins;
  IH_CUDA(c, cudaMemsetAsync(d, 0, sizeof(double) * (4 * bins + 4 + 24), c->stream));
  const size_t hsm = sizeof(double) * bins;
  const unsigned gm = grid_for(M, 256, 8);
  if (!psi_ready) IH_TRY((fft_r2c<T>(c, yfl + 2 * N, 0, spec + 5 * M, 0, 1)));
  k_power_spectrum<T><<<gm, 256, hsm, c->stream>>>(spec + 5 * M, g, d + bins);
  IH_TRY(check_launch(c, "k_power_spectrum"));
  k_lap_spectrum<T><<<gm, 256, 0, c->stream>>>(spec + 5 * M, spec + 6 * M, g);
  IH_TRY(check_launch(c, "k_lap_spectrum"));
  return fft_c2r<T>(c, spec + 6 * M, 0, (T *)c->rbuf[3], 0, 1);
}

// output_post: phi and rho power spectra, constraints, summaries, GW spectrum
// (after the reductions; spec[4] = phihat is free once phi_ps is binned).
template <typename T>
static int output_post(Ctx *c, const Vec &y, const Vec *smry_src) {
  const Geom &g = c->g;
  const long long M = g.M, N = g.N;
  C2<T> *spec = (C2<T> *)c->spec[0];
  T *rho = (T *)c->rbuf[2], *lappsi = (T *)c->rbuf[3];
  const T *yfl = (const T *)y.fl;
  double *d = c->diag;
  const int bins = g.bins;
  const size_t hsm = sizeof(double) * bins;
  const unsigned gm = grid_for(M, 256, 8);
  k_power_spectrum<T><<<gm, 256, hsm, c->stream>>>(spec + 4 * M, g, d);
  IH_TRY(check_launch(c, "k_power_spectrum"));
  IH_TRY((fft_r2c<T>(c, rho, 0, spec + 4 * M, 0, 1)));
  k_power_spectrum<T><<<gm, 256, hsm, c->stream>>>(spec + 4 * M, g, d + 2 * bins);
  IH_TRY(check_launch(c, "k_power_spectrum"));
  double *means = d + 4 * bins + 28;  // [phi_mean, dphi_mean]
  const int nb = nblk_reduce(N);
  for (int s = 0; s < 2; ++s) {
    IH_TRY(mean_into<T>(c, yfl + s * N, N, means + s));
    k_add_scalar<<<1, 1, 0, c->stream>>>(means + s, y.sc + s);
    IH_TRY(check_launch(c, "k_add_scalar"));
  }
  k_constraints<T><<<nb, 256, 0, c->stream>>>(yfl, y.sc, lappsi, rho, c->rs, means, N,
                                              c->partials);
  IH_TRY(check_launch(c, "k_constraints"));
  k_constraints_finish<<<1, 256, 0, c->stream>>>(c->partials, nb, N, d + 4 * bins);
  IH_TRY(check_launch(c, "k_constraints_finish"));
  // summaries: phi, dphi, psi, dpsi of the summary source, then rho and p
  const Vec &src = smry_src ? *smry_src : y;
  IH_CUDA(c, cudaMemcpyAsync(c->hpin, c->rs, sizeof(RhsScalars), cudaMemcpyDeviceToHost,
                             c->stream));
  IH_CUDA(c, cudaMemcpyAsync(c->hpin + 32, src.sc, sizeof(double) * kSc,
                             cudaMemcpyDeviceToHost, c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  RhsScalars rs_h;
  double sc_h[kSc];
  memcpy(&rs_h, c->hpin, sizeof rs_h);
  memcpy(sc_h, c->hpin + 32, sizeof sc_h);
  const T *sfl = (const T *)src.fl;
  for (int s = 0; s < 4; ++s)
    IH_TRY(summary<T>(c, sfl + s * N, nullptr, sc_h[s], N, d + 4 * bins + 4 + 4 * s));
  IH_TRY(summary<T>(c, rho, nullptr, rs_h.rho_bar, N, d + 4 * bins + 4 + 16));
  IH_TRY(summary<T>(c, (const T *)c->rbuf[1], nullptr, rs_h.p_bar, N, d + 4 * bins + 4 + 20));
  if (c->p.enable_gw) {
    k_gw_spectrum<T><<<gm, 256, hsm, c->stream>>>(yfl, c->rs, g, pow(0.01, 1.0 / 3.0),
                                                 d + 3 * bins);
    IH_TRY(check_launch(c, "k_gw_spectrum"));
  }
  c->have_output = 1;
  return IH_OK;
}

int read_output(Ctx *c, ih_output *out) {
  if (!c->have_output) {
    c->err = "no RHS with the output flag has run";
    return IH_ERR_STATE;
  }
  const int bins = c->g.bins;
  std::vector<double> h(4 * bins + 28);
  IH_CUDA(c, cudaMemcpyAsync(h.data(), c->diag, sizeof(double) * h.size(),
                             cudaMemcpyDeviceToHost, c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  if (out->phi_ps) memcpy(out->phi_ps, h.data(), sizeof(double) * bins);
  if (out->psi_ps) memcpy(out->psi_ps, h.data() + bins, sizeof(double) * bins);
  if (out->rho_ps) memcpy(out->rho_ps, h.data() + 2 * bins, sizeof(double) * bins);
  if (out->gw) memcpy(out->gw, h.data() + 3 * bins, sizeof(double) * bins);
  memcpy(out->cstr, h.data() + 4 * bins, sizeof(double) * 4);
  memcpy(out->smry, h.data() + 4 * bins + 4, sizeof(double) * 24);
  return IH_OK;
}

// ---------------------------------------------------------------------------
// The z part of the RHS for grids with a radix-3 factor, unfused: 4 c2r
// passes (d/dx, d/dy, d/dz into the scratch, the laplacian into lap), one
// pointwise pass (rho, p, their FP64 block sums, the six GW products d_i phi
// d_j phi written over the derivatives and into the rest of the scratch) and
// 6 r2c passes -- the same quantities as the fused pass (toolbox.c:129-250,
// 410-424).
template <typename T, bool MIXED>
__global__ void k_pointwise_g(const T *__restrict__ yfl, const double *ysc, T *g0, T *g1, T *g2,
                              T *g3, T *g4, T *g5, T *pout, T *rhoout, int gw, long long N,
                              double mass, double *partials) {
  const double a_sc = ysc[4];
  const T inv_a2 = (T)(1.0 / (a_sc * a_sc));
  const T m2 = (T)(mass * mass);
  const T third = (T)(1.0 / 3.0);
  const T phib = (T)ysc[0], pib = (T)ysc[1], psib = (T)ysc[2];
  double sr = 0.0, sp = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    const T dx = g0[i], dy = g1[i], dz = g2[i];
    T rho, p;
    rho_p<T, MIXED>(dx, dy, dz, yfl[i], yfl[N + i], yfl[2 * N + i], inv_a2, m2, third, phib, pib,
                    psib, rho, p);
    pout[i] = p;
    if (rhoout) rhoout[i] = rho;
    sr += (double)rho;
    sp += (double)p;
    if (gw) {
      g0[i] = dx * dx;
      g1[i] = dx * dy;
      g2[i] = dx * dz;
      g3[i] = dy * dy;
      g4[i] = dy * dz;
      g5[i] = dz * dz;
    }
  }
  sr = block_sum(sr);
  sp = block_sum(sp);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = sr;
    partials[2 * blockIdx.x + 1] = sp;
  }
}

template <typename T>
static int z_pass_generic(Ctx *c, C2<T> *spec, const T *yfl, const double *ysc, T *lap, T *p,
                          T *rho, int *nblk_out) {
  const Geom &g = c->g;
  const long long N = g.N, M = g.M;
  T *gs = (T *)c->gscratch;
  const int gw = c->p.enable_gw;
  IH_TRY((fft_zc2r<T>(c, spec, M, gs, N, 3)));
  IH_TRY((fft_zc2r<T>(c, spec + 3 * M, M, lap, N, 1)));
  unsigned nb = grid_for(N, 256, 4);
  if (2LL * nb > c->partials_cap) nb = (unsigned)(c->partials_cap / 2);
  prof_begin(c, KK_Z_RHS_FUSED);
  if (c->mixed)
    k_pointwise_g<T, true><<<nb, 256, 0, c->stream>>>(yfl, ysc, gs, gs + N, gs + 2 * N, gs + 3 * N,
                                                      gs + 4 * N, gs + 5 * N, p, rho, gw, N,
                                                      g.mass, c->partials);
  else
    k_pointwise_g<T, false><<<nb, 256, 0, c->stream>>>(yfl, ysc, gs, gs + N, gs + 2 * N,
                                                       gs + 3 * N, gs + 4 * N, gs + 5 * N, p, rho,
                                                       gw, N, g.mass, c->partials);
  prof_end(c, KK_Z_RHS_FUSED, (6.0 + (gw ? 6.0 : 0.0) + (rho ? 1.0 : 0.0)) * N * sizeof(T));
  IH_TRY(check_launch(c, "k_pointwise_g"));
  *nblk_out = (int)nb;
  if (gw) {  // xx, xy, xz, yy -> spec[0..3]; yz, zz -> spec[5], spec[6]
    IH_TRY((fft_zr2c<T>(c, gs, N, spec, M, 4)));
    IH_TRY((fft_zr2c<T>(c, gs + 4 * N, N, spec + 5 * M, M, 2)));
  }
  return IH_OK;
}

// ---------------------------------------------------------------------------
// the RHS
template <typename T>
static int rhs_t(Ctx *c, Vec &y, Vec &k, int filter, int output, const Vec *smry_src,
                 const NextLin *next) {
  const Geom &g = c->g;
  const long long N = g.N, M = g.M;
  C2<T> *spec = (C2<T> *)c->spec[0];
  T *yfl = (T *)y.fl, *kfl = (T *)k.fl;
  T *lap = (T *)c->rbuf[0], *p = (T *)c->rbuf[1], *rho = (T *)c->rbuf[2];
  c->calls_rhs += 1;
  // the diagnostics stay those of the last RHS run with the output flag
  if (output == 1) c->have_output = 0;
  const int do_filter = (filter == 1) && c->p.enable_filter;
  // without the filter and the output flag nothing needs the full spectrum
  // of phi: the derivatives come from round trips along x and y on its z
  // spectrum Z (spec[4]), the z parts from Z inside the fused z pass
  const int use_rt = c->roundtrip && c->g.pow2 && !do_filter && output != 1;
  const unsigned gm = grid_for(M, 256, 4);
  // 1. phihat (and with the filter: dphi, psi, dpsi spectra, mask, write back)
  if (do_filter) {
    // spec[4] <- phi, spec[1..3] <- dphi, psi, dpsi
    IH_TRY((fft_r2c<T>(c, yfl, 0, spec + 4 * M, 0, 1)));
    IH_TRY((fft_r2c<T>(c, yfl + N, N, spec + M, M, 3)));
    prof_begin(c, KK_FILTER);
    if (c->mixed)
      k_filter_spectra<T, true><<<gm, 256, 0, c->stream>>>(spec, (const T *)c->mask, M,
                                                           1.0 / (double)N, output, y.sc);
    else
      k_filter_spectra<T, false><<<gm, 256, 0, c->stream>>>(spec, (const T *)c->mask, M,
                                                            1.0 / (double)N, output, y.sc);
    prof_end(c, KK_FILTER, (double)M * (9 + (output ? 1 : 0)) * sizeof(C2<T>) + (double)M * sizeof(T));
    IH_TRY(check_launch(c, "k_filter_spectra"));
    IH_TRY((fft_c2r<T>(c, spec, M, yfl, N, 4)));
  } else if (use_rt) {
    IH_TRY((fft_zr2c<T>(c, yfl, 0, spec + 4 * M, 0, 1)));
  } else {
    IH_TRY((fft_r2c<T>(c, yfl, 0, spec + 4 * M, 0, 1)));
  }
  if (output == 1) IH_TRY(output_pre<T>(c, y, do_filter));
  // 2. derivative spectra in (x, y, kz): d/dx, d/dy, (d/dz), laplacian
  if (use_rt) {
    IH_TRY((fft_xy_roundtrip<T>(c, spec + 4 * M, spec, spec + 3 * M, 0)));
    IH_TRY((fft_xy_roundtrip<T>(c, spec + 4 * M, spec + M, spec + 3 * M, 1)));
  } else {
    IH_TRY((fft_x_deriv4_inv<T>(c, spec + 4 * M, spec, M)));
    IH_TRY((fft_xy<T>(c, spec, M, 4, 1, +1)));
  }
  // 3. fused inverse z + pointwise + GW products forward z (the products
  // plane-major where the one-pass plane transforms take them)
  const int plane = sizeof(T) == 4 && c->gw_plane && !next && gw_plane_ok(c);
  int nblk = 0;
  if (c->g.pow2)
    IH_TRY((fft_z_rhs_fused<T>(c, spec, yfl, y.sc, lap, p, output == 1 ? rho : nullptr,
                               plane ? (C2<T> *)c->gwbuf : spec, c->p.enable_gw, c->partials,
                               &nblk, use_rt, plane)));
  else
    IH_TRY((z_pass_generic<T>(c, spec, yfl, y.sc, lap, p, output == 1 ? rho : nullptr, &nblk)));
  k_reduce_finish<<<1, 256, 0, c->stream>>>(c->partials, nblk, g, y.sc, k.sc, c->rs, c->mixed);
  IH_TRY(check_launch(c, "k_reduce_finish"));
  // 4. diagnostics that need <rho> and H
  if (output == 1) IH_TRY(output_post<T>(c, y, smry_src));
  // 5. tensor modes
  if (c->p.enable_gw) {
    // S_ij spectra: spec[0..3] and spec[5..6]; forward y and x passes
    // (batched: per-array y-then-x ordering measured slower, no L2 reuse;
    // kz slabs of all six arrays where the autotuner chose them)
    if (plane && c->gw_plane == 3) {
      IH_TRY(gw_tt_plane(c, c->gwbuf));
      IH_TRY(update_h_tt(c, c->gwbuf, yfl, kfl, k.sc));
    } else if (plane) {
      IH_TRY(gw_plane_fft(c, c->gwbuf, c->gw_plane));
      IH_TRY(update_h_plane(c, c->gwbuf, yfl, kfl, k.sc));
    } else if (c->gw_slab > 0 && !c->tensor_fused && g.pow2) {
      IH_TRY((fft_gw_yx<T>(c, spec, c->gw_slab)));
      IH_TRY(tensor_last_pass(c, spec, yfl, kfl, k.sc, next, true));
    } else {
      IH_TRY((fft_xy<T>(c, spec, M, 4, 1, -1)));
      IH_TRY((fft_xy<T>(c, spec + 5 * M, M, 2, 1, -1)));
      IH_TRY(tensor_last_pass(c, spec, yfl, kfl, k.sc, next));
    }
  }
  // 6. phi/psi equations of motion (and the next stage input)
  prof_begin(c, KK_UPDATE_PHI_PSI);
  NextLin none{};
  none.skip_pos = c->skip_pos;
  const NextLin &nl = next ? *next : none;
  const unsigned gu = grid_for(N / VecW<T>::W, 256, 4);
  if (c->mixed) {
    if (next)
      k_update_phi_psi<T, true, true><<<gu, 256, 0, c->stream>>>(yfl, y.sc, lap, p, kfl, c->rs, N,
                                                                 g.mass, nl);
    else
      k_update_phi_psi<T, true, false><<<gu, 256, 0, c->stream>>>(yfl, y.sc, lap, p, kfl, c->rs, N,
                                                                  g.mass, nl);
  } else {
    if (next)
      k_update_phi_psi<T, false, true><<<gu, 256, 0, c->stream>>>(yfl, y.sc, lap, p, kfl, c->rs,
                                                                  N, g.mass, nl);
    else
      k_update_phi_psi<T, false, false><<<gu, 256, 0, c->stream>>>(yfl, y.sc, lap, p, kfl, c->rs,
                                                                   N, g.mass, nl);
  }
  prof_end(c, KK_UPDATE_PHI_PSI,
           ((nl.skip_pos ? 8.0 : 10.0) + (next ? 4.0 * (next->n + 2) : 0.0)) * N * sizeof(T));
  IH_TRY(check_launch(c, "k_update_phi_psi"));
  if (next) {
    k_next_sc<<<1, 32, 0, c->stream>>>(*next, k.sc, y.sc);
    IH_TRY(check_launch(c, "k_next_sc"));
  }
  return IH_OK;
}

int rhs(Ctx *c, double t, Vec &y, Vec &k, int filter, int output, const Vec *smry_src,
        const NextLin *next) {
  (void)t;
  if (c->mixed) return rhs_t<float>(c, y, k, filter, output, smry_src, next);
  return rhs_t<double>(c, y, k, filter, output, smry_src, next);
}

int get_field(Ctx *c, int which, double *dev_out) {
  // per-point fields of the last RHS as FP64 full values
  const Geom &g = c->g;
  if (which < 0 || which > 3) {
    c->err = "field index out of range";
    return IH_ERR_ARG;
  }
  if (which == 3) {
    c->err = "the squared gradient is not kept by the fused RHS";
    return IH_ERR_ARG;
  }
  const int src = which == 0 ? 2 : (which == 1 ? 1 : 0);
  // homogeneous parts: rho_bar / p_bar from the RHS scalars
  IH_CUDA(c, cudaMemcpyAsync(&c->rs_host, c->rs, sizeof(RhsScalars), cudaMemcpyDeviceToHost,
                             c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  const double add = which == 0 ? c->rs_host.rho_bar : (which == 1 ? c->rs_host.p_bar : 0.0);

  return convert_add(c, c->rbuf[src], add, g.N, dev_out);
}

template <typename T>
__global__ void k_convert_add(const T *a, double add, long long n, double *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = add + (double)a[i];
}
int convert_add(Ctx *c, const void *a, double add, long long n, double *out) {
  if (c->mixed)
    k_convert_add<float><<<grid_for(n, 256, 4), 256, 0, c->stream>>>((const float *)a, add, n, out);
  else
    k_convert_add<double><<<grid_for(n, 256, 4), 256, 0, c->stream>>>((const double *)a, add, n,
                                                                         out);
  return check_launch(c, "k_convert_add");
}

// fft / ifft of FP64 device buffers in the context precision
template <typename T>
__global__ void k_cast(const double *a, T *b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = (T)a[i];
}
template <typename T>
__global__ void k_uncast(const T *a, double *b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

template <typename T>
static int fft_any_t(Ctx *c, const double *in, double *out_c) {
  const Geom &g = c->g;
  T *r = (T *)c->rbuf[3];
  C2<T> *s = (C2<T> *)c->spec[0] + 6 * g.M;
  k_cast<T><<<grid_for(g.N, 256, 4), 256, 0, c->stream>>>(in, r, g.N);
  IH_TRY(check_launch(c, "k_cast"));
  IH_TRY(fft_r2c<T>(c, r, 0, s, 0, 1));
  k_uncast<T><<<grid_for(2 * g.M, 256, 4), 256, 0, c->stream>>>((const T *)s, out_c, 2 * g.M);
  return check_launch(c, "k_uncast");
}
template <typename T>
static int ifft_any_t(Ctx *c, const double *in_c, double *out) {
  const Geom &g = c->g;
  T *r = (T *)c->rbuf[3];
  C2<T> *s = (C2<T> *)c->spec[0] + 6 * g.M;
  k_cast<T><<<grid_for(2 * g.M, 256, 4), 256, 0, c->stream>>>(in_c, (T *)s, 2 * g.M);
  IH_TRY(check_launch(c, "k_cast"));
  IH_TRY(fft_c2r<T>(c, s, 0, r, 0, 1));
  k_uncast<T><<<grid_for(g.N, 256, 4), 256, 0, c->stream>>>(r, out, g.N);
  return check_launch(c, "k_uncast");
}
int fft_any(Ctx *c, const double *in, double *out_c) {
  return c->mixed ? fft_any_t<float>(c, in, out_c) : fft_any_t<double>(c, in, out_c);
}
int ifft_any(Ctx *c, const double *in_c, double *out) {
  return c->mixed ? ifft_any_t<float>(c, in_c, out) : ifft_any_t<double>(c, in_c, out);
}

// ---------------------------------------------------------------------------
// seeded fluctuation initial conditions (generator shared with the oracle)
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform01(uint64_t key, uint64_t ctr) {
  uint64_t r = mix64(key ^ mix64(ctr));
  return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
__device__ __forceinline__ void normal_pair(uint64_t key, uint64_t idx, double *g1, double *g2) {
  double u1 = uniform01(key, 2 * idx), u2 = uniform01(key, 2 * idx + 1);
  double r = sqrt(-2.0 * log(u1));
  double sn, cs;
  sincos(kTwoPi * u2, &sn, &cs);
  *g1 = r * cs;
  *g2 = r * sn;
}

template <typename T>
__global__ void k_ic_spectra(C2<T> *cphi, C2<T> *cdphi, Geom g, uint64_t key, double amp,
                             double kcut) {
  const double vol = g.lx * g.ly * g.lz, m2 = g.mass * g.mass;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < g.M;
       id += (long long)gridDim.x * blockDim.x) {
    Mode m = mode_of(id, g);
    double re = 0.0, im = 0.0, omega = 0.0;
    const double q = ksq64(g, m.i, m.j, m.k);
    if (id != 0 && q <= kcut * kcut) {
      omega = sqrt(q + m2);
      const double sigma = amp / sqrt(2.0 * omega * vol);
      const bool self_plane = (m.k == 0) || (2 * m.k == g.nz);
      const int pi = (g.nx - m.i) % g.nx, pj = (g.ny - m.j) % g.ny;
      const long long pid = ((long long)pi * g.ny + pj) * g.mz + m.k;
      double g1, g2;
      if (self_plane && pid == id) {
        normal_pair(key, id, &g1, &g2);
        re = sigma * g1;
      } else if (self_plane && pid < id) {
        normal_pair(key, pid, &g1, &g2);
        re = sigma * g1 / sqrt(2.0);
        im = -sigma * g2 / sqrt(2.0);
      } else {
        normal_pair(key, id, &g1, &g2);
        re = sigma * g1 / sqrt(2.0);
        im = sigma * g2 / sqrt(2.0);
      }
    }
    cphi[id] = mk2c<T>((T)re, (T)im);
    cdphi[id] = mk2c<T>((T)(omega * im), (T)(-omega * re));
  }
}
template <typename T>
__global__ void k_ic_finish(T *fl, double *sc, long long N, long long Nf, double phi0,
                            double dphi0, double a0, int mixed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < Nf;
       i += (long long)gridDim.x * blockDim.x) {
    if (i < N) {
      if (!mixed) fl[i] += (T)phi0;
    } else if (i < 2 * N) {
      if (!mixed) fl[i] += (T)dphi0;
    } else {
      fl[i] = (T)0;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc[0] = mixed ? phi0 : 0.0;
    sc[1] = mixed ? dphi0 : 0.0;
    sc[2] = sc[3] = 0.0;
    sc[4] = a0;
    sc[5] = sc[6] = sc[7] = 0.0;
  }
}

template <typename T>
static int ic_t(Ctx *c, uint64_t seed, double phi0, double dphi0, double a0, double amp,
                double kcut) {
  const Geom &g = c->g;
  C2<T> *spec = (C2<T> *)c->spec[0];
  // key = mix64(seed), as the oracle does
  uint64_t z = seed + 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  const uint64_t key = z ^ (z >> 31);
  k_ic_spectra<T><<<grid_for(g.M, 256, 4), 256, 0, c->stream>>>(spec, spec + g.M, g, key, amp,
                                                                kcut);
  IH_TRY(check_launch(c, "k_ic_spectra"));
  T *fl = (T *)c->y.fl;
  IH_TRY(fft_c2r<T>(c, spec, g.M, fl, g.N, 2));
  k_ic_finish<T><<<grid_for(g.Nf, 256, 4), 256, 0, c->stream>>>(fl, c->y.sc, g.N, g.Nf, phi0,
                                                               dphi0, a0, c->mixed);
  return check_launch(c, "k_ic_finish");
}

int ic_fluctuations(Ctx *c, uint64_t seed, double phi0, double dphi0, double a0, double amp,
                    double kcut) {
  if (c->mixed) return ic_t<float>(c, seed, phi0, dphi0, a0, amp, kcut);
  return ic_t<double>(c, seed, phi0, dphi0, a0, amp, kcut);
}

// mk_initial_psi (setup.c:825-903).  The spectra of (phi - <phi>) and
// (dphi - <dphi>) differ from those of phi and dphi only at k = 0, which the
// solve sets to zero, so the fluctuation arrays are transformed directly.
template <typename T>
__global__ void k_psi_spectrum(const C2<T> *dphic, const C2<T> *phic, C2<T> *out, Geom g,
                               const double *means, const RhsScalars *rs) {
  const double dphi_mean = means[1], ddphi_mean = means[2];
  const double a2 = rs->a2;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < g.M;
       id += (long long)gridDim.x * blockDim.x) {
    if (id == 0) {
      out[0] = mk2c<T>(0, 0);
      continue;
    }
    Mode m = mode_of(id, g);
    const double den = (-dphi_mean * dphi_mean + 2.0 * ksq64(g, m.i, m.j, m.k) / a2) * (double)g.N;
    C2<T> a = dphic[id], b = phic[id];
    out[id] = mk2c<T>((T)((-dphi_mean * (double)a.x + ddphi_mean * (double)b.x) / den),
                      (T)((-dphi_mean * (double)a.y + ddphi_mean * (double)b.y) / den));
  }
}
template <typename T>
__global__ void k_dpsi_init(T *fl, const double *sc, const double *means, const RhsScalars *rs,
                            long long N) {
  // dpsi = 1/2 <dphi> (phi - <phi>) - H psi (setup.c:860-863)
  const double dphi_mean = means[1], phi_mean = means[0], H = rs->H;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    const double ph = sc[0] + (double)fl[i];
    fl[3 * N + i] = (T)(0.5 * dphi_mean * (ph - phi_mean) - H * (double)fl[2 * N + i]);
  }
}
__global__ void k_zero_psi_scalars(double *sc) { sc[2] = sc[3] = 0.0; }

template <typename T>
static int initial_psi_t(Ctx *c) {
  const Geom &g = c->g;
  const long long N = g.N, M = g.M;
  T *fl = (T *)c->y.fl;
  IH_CUDA(c, cudaMemsetAsync(fl + 2 * N, 0, sizeof(T) * 2 * N, c->stream));
  k_zero_psi_scalars<<<1, 1, 0, c->stream>>>(c->y.sc);
  IH_TRY(check_launch(c, "k_zero_psi_scalars"));
  // the RHS with filter = output = 0 into k[1] (the reference writes dfield)
  IH_TRY(rhs(c, c->t, c->y, c->k[1], 0, 0, nullptr));
  double *means = c->diag + 4 * g.bins + 40;  // [phi_mean, dphi_mean, ddphi_mean]
  const void *srcs[3] = {fl, fl + N, (T *)c->k[1].fl + N};
  const double *adds[3] = {c->y.sc + 0, c->y.sc + 1, c->k[1].sc + 1};
  const int nb = nblk_reduce(N);
  for (int s = 0; s < 3; ++s) {
    k_partial_sum<T><<<nb, 256, 0, c->stream>>>((const T *)srcs[s], N, c->partials);
    IH_TRY(check_launch(c, "k_partial_sum"));
    k_finish_sum<<<1, 256, 0, c->stream>>>(c->partials, nb, 1.0 / (double)N, 0.0, means + s);
    IH_TRY(check_launch(c, "k_finish_sum"));
    k_add_scalar<<<1, 1, 0, c->stream>>>(means + s, adds[s]);
    IH_TRY(check_launch(c, "k_add_scalar"));
  }
  C2<T> *spec = (C2<T> *)c->spec[0];
  IH_TRY(fft_r2c<T>(c, fl + N, 0, spec, 0, 1));        // dphi -> spec[0]
  IH_TRY(fft_r2c<T>(c, fl, 0, spec + M, 0, 1));        // phi  -> spec[1]
  k_psi_spectrum<T><<<grid_for(M, 256, 4), 256, 0, c->stream>>>(spec, spec + M, spec + 2 * M, g,
                                                               means, c->rs);
  IH_TRY(check_launch(c, "k_psi_spectrum"));
  IH_TRY(fft_c2r<T>(c, spec + 2 * M, 0, fl + 2 * N, 0, 1));
  k_dpsi_init<T><<<grid_for(N, 256, 4), 256, 0, c->stream>>>(fl, c->y.sc, means, c->rs, N);
  return check_launch(c, "k_dpsi_init");
}

int initial_psi(Ctx *c) {
  return c->mixed ? initial_psi_t<float>(c) : initial_psi_t<double>(c);
}

int mask_init(Ctx *c, void *mask) {
  if (c->mixed)
    k_mask_init<float><<<grid_for(c->g.M, 256, 4), 256, 0, c->stream>>>((float *)mask, c->g);
  else
    k_mask_init<double><<<grid_for(c->g.M, 256, 4), 256, 0, c->stream>>>((double *)mask, c->g);
  return check_launch(c, "k_mask_init");
}

}  // namespace ih
