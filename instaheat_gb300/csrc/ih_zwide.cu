// ih_zwide.cu -- the fused last z pass of the RHS for nz = 256 (H = 128
// complex points per row), on a wide-row FFT engine; FP32 (mixed form) and
// FP64 (plain form) instantiations of the same code.
//
// The general z engine (ih_fft.cu) spreads one row over a whole warp (32
// lanes x H/32 values) and spends most of its instructions on five shuffle
// stages per transform.  Here a row lives on 8 lanes with 16 values each, 4
// rows per warp:
//   H = 16 x 8, lane t of a row group holds Z[t + 8m] (m < 16);
//   inverse: a 16-point DFT in registers over m, the twiddle w^(p t),
//            one shared-memory transpose (columns swizzled t ^ (p >> 1) so
//            that the 8 lanes of a group always hit 8 different bank pairs),
//            two 8-point DFTs in registers: lane t ends with z[2t + e + 16q]
//            (e < 2, q < 8), i.e. the reals 4t + 32q .. 4t + 32q + 3 -- one
//            float4 per q, so the pointwise loads and stores are float4s;
//   forward: the same steps in reverse order from that layout.
// The c2r input pairs X_k with X_(H-k): lane t loads both straight from the
// row (the partner line is in L1), so the pre-processing needs no exchange;
// the r2c output pairs Z_k with Z_(H-k) by one shuffle per register from lane
// 8 - t (lane 0 pairs its own registers).  d/dx and d/dy of phi stay in a
// thread-private shared-memory slab between the inverse transforms and the
// products; d/dz stays in registers.
//
// Same inputs, outputs and partial sums as k_fft_z_rhs_fused (see there and
// toolbox.c:172-250, 311-346).  In FP64 the engine's point is arithmetic, not
// memory: every butterfly runs in registers (16- and 8-point DFTs and one
// shared-memory transpose) where the warp-row engine spends five of its seven
// radix-2 stages on shuffle exchanges that multiply every lane's value by a
// twiddle, and the plain FP64 form is bound by the FP64 pipe.
#include "ih_internal.cuh"
#include "ih_fftcore.cuh"

namespace ih {
namespace {

constexpr int kH = 128;              // complex points per row
constexpr int kRowsW = 4;            // rows per warp (8 lanes each)
constexpr int kWarpsW = 4;           // warps per CTA
constexpr int kXch = 16 * 8 + 8;     // transpose scratch per row (complex), padded so that
                                     // the row groups of a warp alternate bank halves

// four consecutive reals of a lane (4t + 32q .. 4t + 32q + 3)
template <typename T> struct Quad;
template <> struct Quad<float> {
  using type = float4;
};
template <> struct Quad<double> {
  struct __align__(16) type {
    double x, y, z, w;
  };
};
template <typename T> using Q4 = typename Quad<T>::type;

template <typename T>
__device__ __forceinline__ Q4<T> q4(const C2<T> &a, const C2<T> &b) {
  Q4<T> r;
  r.x = a.x;
  r.y = a.y;
  r.z = b.x;
  r.w = b.y;
  return r;
}

template <typename T> struct WideSmem {
  C2<T> twh[kH];                     // exp(-2 pi i k/H)
  C2<T> twz[2 * kH];                 // exp(-2 pi i k/nz)
  C2<T> xch[kWarpsW][kRowsW][kXch];
  Q4<T> grad[kWarpsW][2][8][32];     // d/dx, d/dy of each lane's 32 points: [q][lane]
  double red[2][kWarpsW];
};
// with the prefetch: each row's next input spectrum row (kH + 1 values)
template <typename T> struct WideSmemPF : WideSmem<T> {
  C2<T> pf[kWarpsW][kRowsW][kH + 1];
};

// lane t: v[m] = Z[t + 8m] -> v[2q + e] = z[2t + e + 16q] (inverse, unnormalised)
template <typename T>
__device__ __forceinline__ void zw_inverse(C2<T> (&v)[16], int t, C2<T> *xch,
                                           const C2<T> *twh) {
  reg_dft<T, 16>(v, twh, kH / 16, +1);
#pragma unroll
  for (int p = 1; p < 16; ++p) {
    C2<T> w = twh[p * t];  // p t < H
    w.y = -w.y;
    v[p] = cmul(v[p], w);
  }
#pragma unroll
  for (int p = 0; p < 16; ++p) xch[p * 8 + (t ^ (p >> 1))] = v[p];
  __syncwarp();
  C2<T> u0[8], u1[8];
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    u0[s] = xch[(2 * t) * 8 + (s ^ t)];
    u1[s] = xch[(2 * t + 1) * 8 + (s ^ t)];
  }
  __syncwarp();
  reg_dft<T, 8>(u0, twh, kH / 8, +1);
  reg_dft<T, 8>(u1, twh, kH / 8, +1);
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    v[2 * q] = u0[q];
    v[2 * q + 1] = u1[q];
  }
}

// lane t: v[2q + e] = z[2t + e + 16q] -> v[m] = Z[t + 8m] (forward)
template <typename T>
__device__ __forceinline__ void zw_forward(C2<T> (&v)[16], int t, C2<T> *xch,
                                           const C2<T> *twh) {
  C2<T> u0[8], u1[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    u0[q] = v[2 * q];
    u1[q] = v[2 * q + 1];
  }
  reg_dft<T, 8>(u0, twh, kH / 8, -1);
  reg_dft<T, 8>(u1, twh, kH / 8, -1);
#pragma unroll
  for (int s = 1; s < 8; ++s) {
    u0[s] = cmul(u0[s], twh[(2 * t) * s]);
    u1[s] = cmul(u1[s], twh[(2 * t + 1) * s]);
  }
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    xch[(2 * t) * 8 + (s ^ t)] = u0[s];
    xch[(2 * t + 1) * 8 + (s ^ t)] = u1[s];
  }
  __syncwarp();
#pragma unroll
  for (int p = 0; p < 16; ++p) v[p] = xch[p * 8 + (t ^ (p >> 1))];
  __syncwarp();
  reg_dft<T, 16>(v, twh, kH / 16, -1);
}

// c2r pre-processing: x[m] = X_k, xp[m] = X_(H-k) (k = t + 8m) ->
// v[m] = E + i O with E = X_k + conj X_(H-k), O = (X_k - conj X_(H-k)) exp(+2 pi i k/nz)
template <typename T>
__device__ __forceinline__ void zw_c2r_prep(const C2<T> (&x)[16], const C2<T> (&xp)[16], int t,
                                            const C2<T> *twz, C2<T> (&v)[16]) {
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const C2<T> pc = mk2<T>(xp[m].x, -xp[m].y);
    const C2<T> e = cadd(x[m], pc), d = csub(x[m], pc);
    C2<T> wn = twz[t + 8 * m];
    wn.y = -wn.y;
    const C2<T> o = cmul(d, wn);
    v[m] = mk2<T>(e.x - o.y, e.y + o.x);
  }
}

// r2c post-processing: v[m] = Z_k (k = t + 8m) -> X_k = E_k + exp(-2 pi i k/nz) O_k,
// E_k = (Z_k + conj Z_(H-k))/2, O_k = (Z_k - conj Z_(H-k))/(2i); xH = X_H on t == 0.
// Z_(H-k) is register 15 - m of lane 8 - t (t > 0) or register (16 - m) mod 16
// of lane 0 itself.
template <typename T>
__device__ __forceinline__ void zw_r2c_post(C2<T> (&v)[16], int t, int gbase, const C2<T> *twz,
                                            C2<T> &xH) {
  C2<T> pz[16];
  const int src = gbase | ((8 - t) & 7);
#pragma unroll
  for (int m = 0; m < 16; ++m) pz[m] = shfl_idx_c(v[15 - m], src);
  if (t == 0) {
#pragma unroll
    for (int m = 0; m < 16; ++m) pz[m] = v[(16 - m) & 15];
  }
  const T half = (T)0.5;
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const C2<T> z = v[m];
    const C2<T> zc = mk2<T>(pz[m].x, -pz[m].y);
    const C2<T> e = mk2<T>(half * (z.x + zc.x), half * (z.y + zc.y));
    const C2<T> o = mk2<T>(half * (z.y - zc.y), -half * (z.x - zc.x));
    if (m == 0) xH = csub(e, o);  // exp(-i pi) = -1
    v[m] = cadd(e, cmul(o, twz[t + 8 * m]));
  }
}

// ZSRC: arrays 0, 1 = d/dx Z, d/dy Z, array 3 = the laplacian (completed by
// the y round trip), array 4 = Z (the z derivative formed here); otherwise
// arrays 0..3 = the four full derivative spectra.
// PF: the four inverse transforms read their rows from shared memory, where
// cp.async copied them while the previous transform ran (the global loads of
// a row are then off the transform's critical path).
// PLANE: the six GW source spectra are written plane-major, S[kz][x][y]
// (row = x ny + y, element kz rows + row), for the one-pass plane transforms
// (ih_gwplane.cu): each warp stages its four rows in its exchange buffer and
// stores eight kz values x four consecutive y per instruction (32-byte runs;
// the four warps of a CTA complete each 128-byte line of a kz plane).
template <typename T, bool ZSRC, bool PLANE, bool PF>
__global__ void __launch_bounds__(32 * kWarpsW, (sizeof(T) == 4 ? (PF ? 3 : 4) : 2)) k_fft_z_rhs_wide(
    const C2<T> *d4, long long dstride, const T *__restrict__ yfl, const double *ysc, T *lap,
    T *pout, T *rhoout, C2<T> *s6, long long sstride4, C2<T> *s6b, int gw, double *partials,
    Geom g, const C2<T> *__restrict__ twhg, const C2<T> *__restrict__ twzg) {
  using V = C2<T>;
  constexpr bool MIXED = sizeof(T) == 4;  // FP32 fields are fluctuations (mixed form)
  extern __shared__ __align__(16) unsigned char smraw[];
  WideSmem<T> &sm = *reinterpret_cast<WideSmem<T> *>(smraw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int t = lane & 7, grp = lane >> 3, gbase = lane & ~7;
  for (int i = tid; i < kH; i += blockDim.x) sm.twh[i] = twhg[i];
  for (int i = tid; i < 2 * kH; i += blockDim.x) sm.twz[i] = twzg[i];
  __syncthreads();
  const long long rows = (long long)g.nx * g.ny;
  const long long row = ((long long)blockIdx.x * kWarpsW + warp) * kRowsW + grp;
  const bool valid = row < rows;
  V *xch = sm.xch[warp][grp];
  const T invnz = (T)(1.0 / (double)g.nz);
  const long long rs = row * (kH + 1);  // first element of the row in a half spectrum

  // PF: the row group's copy of its next input row (lane t copies k = t + 8j)
  V *pfrow = nullptr;
  if constexpr (PF) pfrow = reinterpret_cast<WideSmemPF<T> &>(sm).pf[warp][grp];
  auto prefetch = [&](int a) {
    const V *ra = d4 + (ZSRC && a == 2 ? 4 : a) * dstride + rs;
#pragma unroll
    for (int j = 0; j <= kH / 8; ++j) {
      const int k = t + 8 * j;
      if (k <= kH) cp_async_c<T>(pfrow + k, valid ? ra + k : d4, valid);
    }
    cp_async_commit();
  };

  // fetch row a (x: X_k, xp: X_(H-k)), pre-process, inverse transform; PF:
  // from the prefetched copy, then start the copy of row `next`
  auto inverse_of = [&](int a, int next, V (&v)[16]) {
    V x[16], xp[16];
    if constexpr (PF) {
      cp_async_wait<0>();
      __syncwarp();  // the other lanes' copies of the row are visible
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        x[m] = pfrow[t + 8 * m];
        xp[m] = pfrow[kH - t - 8 * m];
      }
      __syncwarp();  // every lane has read the row before it is overwritten
      if (next >= 0) prefetch(next);
    } else {
      const V *ra = d4 + (ZSRC && a == 2 ? 4 : a) * dstride + rs;
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        x[m] = valid ? ra[t + 8 * m] : mk2<T>(0, 0);
        xp[m] = valid ? ra[kH - t - 8 * m] : mk2<T>(0, 0);
      }
    }
    if (ZSRC && a == 2) {  // i kz Z / nz, zero on the Nyquist index
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const int k = t + 8 * m, kp = kH - k;
        const T f = kfac<T>(g.kzu, k) * invnz;
        const T fp = (kp == kH) ? (T)0 : kfac<T>(g.kzu, kp) * invnz;
        x[m] = mk2<T>(-x[m].y * f, x[m].x * f);
        xp[m] = mk2<T>(-xp[m].y * fp, xp[m].x * fp);
      }
    }
    zw_c2r_prep<T>(x, xp, t, sm.twz, v);
    zw_inverse<T>(v, t, xch, sm.twh);
  };

  const long long N = g.N;
  const long long e0 = row * (2 * kH) + 4 * t;  // first real of the lane in the row
  // the four inverse transforms in one loop (one copy of the transform code:
  // the kernel's instruction footprint): the laplacian is written out, d/dx
  // and d/dy go to the shared slab, d/dz stays in registers
  V dz[16];
  if constexpr (PF) prefetch(3);
#pragma unroll 1
  for (int i = 0; i < 4; ++i) {
    const int a = (i + 3) & 3;  // 3, 0, 1, 2
    V v[16];
    inverse_of(a, i < 3 ? (i + 4) & 3 : -1, v);
    if (a == 3) {
      if (valid) {
#pragma unroll
        for (int q = 0; q < 8; ++q)
          *reinterpret_cast<Q4<T> *>(lap + e0 + 32 * q) = q4<T>(v[2 * q], v[2 * q + 1]);
      }
    } else if (a < 2) {
#pragma unroll
      for (int q = 0; q < 8; ++q) sm.grad[warp][a][q][lane] = q4<T>(v[2 * q], v[2 * q + 1]);
    } else {
#pragma unroll
      for (int m = 0; m < 16; ++m) dz[m] = v[m];
    }
  }

  // 4. pointwise energy density and pressure, FP64 partial sums
  const double a_sc = ysc[4];
  const T inv_a2 = (T)(1.0 / (a_sc * a_sc));
  const T m2 = (T)(g.mass * g.mass);
  const T third = (T)(1.0 / 3.0);
  const T phib = (T)ysc[0], pib = (T)ysc[1], psib = (T)ysc[2];
  double dr = 0.0, dp = 0.0;
  if (valid) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const long long e = e0 + 32 * q;
      const Q4<T> ph = *reinterpret_cast<const Q4<T> *>(yfl + e);
      const Q4<T> dph = *reinterpret_cast<const Q4<T> *>(yfl + N + e);
      const Q4<T> ps = *reinterpret_cast<const Q4<T> *>(yfl + 2 * N + e);
      const Q4<T> gx = sm.grad[warp][0][q][lane], gy = sm.grad[warp][1][q][lane];
      const Q4<T> gz = q4<T>(dz[2 * q], dz[2 * q + 1]);
      Q4<T> r4, p4;
      rho_p<T, MIXED>(gx.x, gy.x, gz.x, ph.x, dph.x, ps.x, inv_a2, m2, third, phib, pib, psib,
                      r4.x, p4.x);
      rho_p<T, MIXED>(gx.y, gy.y, gz.y, ph.y, dph.y, ps.y, inv_a2, m2, third, phib, pib, psib,
                      r4.y, p4.y);
      rho_p<T, MIXED>(gx.z, gy.z, gz.z, ph.z, dph.z, ps.z, inv_a2, m2, third, phib, pib, psib,
                      r4.z, p4.z);
      rho_p<T, MIXED>(gx.w, gy.w, gz.w, ph.w, dph.w, ps.w, inv_a2, m2, third, phib, pib, psib,
                      r4.w, p4.w);
      *reinterpret_cast<Q4<T> *>(pout + e) = p4;
      if (rhoout) *reinterpret_cast<Q4<T> *>(rhoout + e) = r4;
      // T over 4 points, FP64 beyond
      dr += (double)((r4.x + r4.y) + (r4.z + r4.w));
      dp += (double)((p4.x + p4.y) + (p4.z + p4.w));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dr += __shfl_down_sync(0xffffffffu, dr, o);
    dp += __shfl_down_sync(0xffffffffu, dp, o);
  }
  if (lane == 0) {
    sm.red[0][warp] = dr;
    sm.red[1][warp] = dp;
  }
  __syncthreads();
  if (tid == 0) {
    double sa = 0.0, sb = 0.0;
#pragma unroll
    for (int w = 0; w < kWarpsW; ++w) {
      sa += sm.red[0][w];
      sb += sm.red[1][w];
    }
    partials[2 * blockIdx.x] = sa;
    partials[2 * blockIdx.x + 1] = sb;
  }
  if (!gw) return;

  // 5. the six GW source products d_i phi d_j phi, forward transforms
#pragma unroll 1
  for (int pr = 0; pr < 6; ++pr) {
    const int ia = pr < 3 ? 0 : (pr < 5 ? 1 : 2);
    const int ib = pr < 3 ? pr : (pr < 5 ? pr - 2 : 2);
    V v[16];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const Q4<T> gq = q4<T>(dz[2 * q], dz[2 * q + 1]);
      const Q4<T> A = ia < 2 ? sm.grad[warp][ia][q][lane] : gq;
      const Q4<T> Bv = ib < 2 ? sm.grad[warp][ib][q][lane] : gq;
      v[2 * q] = mk2<T>(A.x * Bv.x, A.y * Bv.y);
      v[2 * q + 1] = mk2<T>(A.z * Bv.z, A.w * Bv.w);
    }
    zw_forward<T>(v, t, xch, sm.twh);
    V xH;
    zw_r2c_post<T>(v, t, gbase, sm.twz, xH);
    if constexpr (PLANE) {
      V *arr = pr < 4 ? s6 + pr * sstride4 : s6b + (pr - 4) * sstride4;
#pragma unroll
      for (int m = 0; m < 16; ++m) xch[t + 8 * m] = v[m];
      if (t == 0) xch[kH] = xH;
      __syncwarp();
      const long long row0 = ((long long)blockIdx.x * kWarpsW + warp) * kRowsW;
      const int gs = lane & 3;
      const V *xs = sm.xch[warp][gs];
#pragma unroll
      for (int q = 0; q < (kH + 1 + 7) / 8; ++q) {
        const int kz = 8 * q + (lane >> 2);
        if (kz <= kH && row0 + gs < rows) arr[(long long)kz * rows + row0 + gs] = xs[kz];
      }
      __syncwarp();
    } else {
      V *dst = (pr < 4 ? s6 + pr * sstride4 : s6b + (pr - 4) * sstride4) + rs;
      if (valid) {
#pragma unroll
        for (int m = 0; m < 16; ++m) dst[t + 8 * m] = v[m];
        if (t == 0) dst[kH] = xH;
      }
    }
  }
}

// Plain r2c z pass on the wide-row engine (the z spectrum of phi in the
// round-trip RHS, the filter's forward transforms): each lane loads its
// reals 4t + 32q .. 4t + 32q + 3 of a row as float4s, one forward transform,
// the r2c split, the row stored (t + 8m per lane, X_H by lane 0).
template <typename T> struct WideR2cSmem {
  C2<T> twh[kH];
  C2<T> twz[2 * kH];
  C2<T> xch[kWarpsW][kRowsW][kXch];
};

template <typename T>
__global__ void __launch_bounds__(32 * kWarpsW) k_fft_zr2c_wide(const T *__restrict__ in,
                                                               long long istride, C2<T> *out,
                                                               long long ostride, long long rows,
                                                               const C2<T> *__restrict__ twhg,
                                                               const C2<T> *__restrict__ twzg) {
  using V = C2<T>;
  __shared__ WideR2cSmem<T> sm;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int t = lane & 7, grp = lane >> 3, gbase = lane & ~7;
  for (int i = tid; i < kH; i += blockDim.x) sm.twh[i] = twhg[i];
  for (int i = tid; i < 2 * kH; i += blockDim.x) sm.twz[i] = twzg[i];
  __syncthreads();
  const long long row = ((long long)blockIdx.x * kWarpsW + warp) * kRowsW + grp;
  const bool valid = row < rows;
  const T *src = in + blockIdx.y * istride + row * (2 * kH) + 4 * t;
  V v[16];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    Q4<T> x;
    if (valid) {
      x = *reinterpret_cast<const Q4<T> *>(src + 32 * q);
    } else {
      x.x = x.y = x.z = x.w = (T)0;
    }
    v[2 * q] = mk2<T>(x.x, x.y);
    v[2 * q + 1] = mk2<T>(x.z, x.w);
  }
  zw_forward<T>(v, t, sm.xch[warp][grp], sm.twh);
  V xH;
  zw_r2c_post<T>(v, t, gbase, sm.twz, xH);
  if (valid) {
    V *dst = out + blockIdx.y * ostride + row * (kH + 1);
#pragma unroll
    for (int m = 0; m < 16; ++m) dst[t + 8 * m] = v[m];
    if (t == 0) dst[kH] = xH;
  }
}

}  // namespace

bool fused_wide_ok(const Ctx *c) {
  return c->zwide && c->g.h == kH;
}

int zr2c_wide_launch(Ctx *c, const void *in, long long istride, void *out, long long ostride,
                     int count) {
  const Geom &g = c->g;
  const long long rows = (long long)g.nx * g.ny;
  const long long per = (long long)kRowsW * kWarpsW;
  const dim3 grid((unsigned)((rows + per - 1) / per), count);
  if (c->mixed)
    k_fft_zr2c_wide<float><<<grid, 32 * kWarpsW, 0, c->stream>>>(
        reinterpret_cast<const float *>(in), istride, reinterpret_cast<float2 *>(out), ostride,
        rows, reinterpret_cast<const float2 *>(c->tw_h), reinterpret_cast<const float2 *>(c->tw_z));
  else
    k_fft_zr2c_wide<double><<<grid, 32 * kWarpsW, 0, c->stream>>>(
        reinterpret_cast<const double *>(in), istride, reinterpret_cast<double2 *>(out), ostride,
        rows, reinterpret_cast<const double2 *>(c->tw_h),
        reinterpret_cast<const double2 *>(c->tw_z));
  return IH_OK;
}

template <typename T, bool ZSRC, bool PLANE, bool PF>
static void wide_launch_pf(Ctx *c, unsigned nblk, const void *d4, long long M, const void *yfl,
                           const double *ysc, void *lap, void *p, void *rho, void *s6, int gw,
                           double *partials, const Geom &g) {
  const size_t sm = PF ? sizeof(WideSmemPF<T>) : sizeof(WideSmem<T>);
  cudaFuncSetAttribute(k_fft_z_rhs_wide<T, ZSRC, PLANE, PF>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  // row layout: the sources in spectra 0..3, 5, 6 of the RHS block; plane
  // layout: six consecutive spectra of their own buffer
  C2<T> *s = reinterpret_cast<C2<T> *>(s6);
  k_fft_z_rhs_wide<T, ZSRC, PLANE, PF><<<nblk, 32 * kWarpsW, sm, c->stream>>>(
      (const C2<T> *)d4, M, (const T *)yfl, ysc, (T *)lap, (T *)p, (T *)rho, s, M,
      s + (PLANE ? 4 : 5) * M, gw, partials, g, reinterpret_cast<const C2<T> *>(c->tw_h),
      reinterpret_cast<const C2<T> *>(c->tw_z));
}

// zwide 2: the prefetching form (FP32 only; the FP64 pass is bound by its
// arithmetic, not by its loads)
template <typename T, bool ZSRC, bool PLANE>
static void wide_launch_t(Ctx *c, unsigned nblk, const void *d4, long long M, const void *yfl,
                          const double *ysc, void *lap, void *p, void *rho, void *s6, int gw,
                          double *partials, const Geom &g) {
  if constexpr (sizeof(T) == 4) {
    if (c->zwide == 2) {
      wide_launch_pf<T, ZSRC, PLANE, true>(c, nblk, d4, M, yfl, ysc, lap, p, rho, s6, gw,
                                           partials, g);
      return;
    }
  }
  wide_launch_pf<T, ZSRC, PLANE, false>(c, nblk, d4, M, yfl, ysc, lap, p, rho, s6, gw, partials,
                                        g);
}

int fused_wide_launch(Ctx *c, const void *d4, const void *yfl, const double *ysc, void *lap,
                      void *p, void *rho, void *s6, int gw, double *partials, int *nblk_out,
                      int zsrc, int plane) {
  const Geom &g = c->g;
  const long long rows = (long long)g.nx * g.ny;
  const long long per = (long long)kRowsW * kWarpsW;
  const unsigned nblk = (unsigned)((rows + per - 1) / per);
  if (2LL * nblk > c->partials_cap) {
    c->err = "grid too large for the RHS partial-sum buffer";
    return IH_ERR_ARG;
  }
  if (plane && !c->mixed) {
    c->err = "plane-major tensor sources are a mixed-form path";
    return IH_ERR_STATE;
  }
  const long long M = g.M;
  if (c->mixed) {
    if (zsrc && plane)
      wide_launch_t<float, true, true>(c, nblk, d4, M, yfl, ysc, lap, p, rho, s6, gw, partials, g);
    else if (zsrc)
      wide_launch_t<float, true, false>(c, nblk, d4, M, yfl, ysc, lap, p, rho, s6, gw, partials, g);
    else if (plane)
      wide_launch_t<float, false, true>(c, nblk, d4, M, yfl, ysc, lap, p, rho, s6, gw, partials, g);
    else
      wide_launch_t<float, false, false>(c, nblk, d4, M, yfl, ysc, lap, p, rho, s6, gw, partials, g);
  } else {
    if (zsrc)
      wide_launch_t<double, true, false>(c, nblk, d4, M, yfl, ysc, lap, p, rho, s6, gw, partials, g);
    else
      wide_launch_t<double, false, false>(c, nblk, d4, M, yfl, ysc, lap, p, rho, s6, gw, partials, g);
  }
  *nblk_out = (int)nblk;
  return IH_OK;
}

}  // namespace ih
