// ih_zwide.cu -- the fused last z pass of the RHS for nz = 256 (H = 128
// complex points per row) in the mixed form, on a wide-row FFT engine.
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
// toolbox.c:172-250, 311-346).
#include "ih_internal.cuh"
#include "ih_fftcore.cuh"

namespace ih {
namespace {

constexpr int kH = 128;              // complex points per row
constexpr int kRowsW = 4;            // rows per warp (8 lanes each)
constexpr int kWarpsW = 4;           // warps per CTA
constexpr int kXch = 16 * 8 + 8;     // transpose scratch per row (complex), padded so that
                                     // the row groups of a warp alternate bank halves

struct WideSmem {
  float2 twh[kH];                    // exp(-2 pi i k/H)
  float2 twz[2 * kH];                // exp(-2 pi i k/nz)
  float2 xch[kWarpsW][kRowsW][kXch];
  float4 grad[kWarpsW][2][8][32];    // d/dx, d/dy of each lane's 32 points: [q][lane]
  double red[2][kWarpsW];
};

// lane t: v[m] = Z[t + 8m] -> v[2q + e] = z[2t + e + 16q] (inverse, unnormalised)
__device__ __forceinline__ void zw_inverse(float2 (&v)[16], int t, float2 *xch,
                                           const float2 *twh) {
  reg_dft<float, 16>(v, twh, kH / 16, +1);
#pragma unroll
  for (int p = 1; p < 16; ++p) {
    float2 w = twh[p * t];  // p t < H
    w.y = -w.y;
    v[p] = cmul(v[p], w);
  }
#pragma unroll
  for (int p = 0; p < 16; ++p) xch[p * 8 + (t ^ (p >> 1))] = v[p];
  __syncwarp();
  float2 u0[8], u1[8];
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    u0[s] = xch[(2 * t) * 8 + (s ^ t)];
    u1[s] = xch[(2 * t + 1) * 8 + (s ^ t)];
  }
  __syncwarp();
  reg_dft<float, 8>(u0, twh, kH / 8, +1);
  reg_dft<float, 8>(u1, twh, kH / 8, +1);
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    v[2 * q] = u0[q];
    v[2 * q + 1] = u1[q];
  }
}

// lane t: v[2q + e] = z[2t + e + 16q] -> v[m] = Z[t + 8m] (forward)
__device__ __forceinline__ void zw_forward(float2 (&v)[16], int t, float2 *xch,
                                           const float2 *twh) {
  float2 u0[8], u1[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    u0[q] = v[2 * q];
    u1[q] = v[2 * q + 1];
  }
  reg_dft<float, 8>(u0, twh, kH / 8, -1);
  reg_dft<float, 8>(u1, twh, kH / 8, -1);
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
  reg_dft<float, 16>(v, twh, kH / 16, -1);
}

// c2r pre-processing: x[m] = X_k, xp[m] = X_(H-k) (k = t + 8m) ->
// v[m] = E + i O with E = X_k + conj X_(H-k), O = (X_k - conj X_(H-k)) exp(+2 pi i k/nz)
__device__ __forceinline__ void zw_c2r_prep(const float2 (&x)[16], const float2 (&xp)[16], int t,
                                            const float2 *twz, float2 (&v)[16]) {
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const float2 pc = make_float2(xp[m].x, -xp[m].y);
    const float2 e = cadd(x[m], pc), d = csub(x[m], pc);
    float2 wn = twz[t + 8 * m];
    wn.y = -wn.y;
    const float2 o = cmul(d, wn);
    v[m] = make_float2(e.x - o.y, e.y + o.x);
  }
}

// r2c post-processing: v[m] = Z_k (k = t + 8m) -> X_k = E_k + exp(-2 pi i k/nz) O_k,
// E_k = (Z_k + conj Z_(H-k))/2, O_k = (Z_k - conj Z_(H-k))/(2i); xH = X_H on t == 0.
// Z_(H-k) is register 15 - m of lane 8 - t (t > 0) or register (16 - m) mod 16
// of lane 0 itself.
__device__ __forceinline__ void zw_r2c_post(float2 (&v)[16], int t, int gbase, const float2 *twz,
                                            float2 &xH) {
  float2 pz[16];
  const int src = gbase | ((8 - t) & 7);
#pragma unroll
  for (int m = 0; m < 16; ++m) pz[m] = shfl_idx_c(v[15 - m], src);
  if (t == 0) {
#pragma unroll
    for (int m = 0; m < 16; ++m) pz[m] = v[(16 - m) & 15];
  }
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const float2 z = v[m];
    const float2 zc = make_float2(pz[m].x, -pz[m].y);
    const float2 e = make_float2(0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y));
    const float2 o = make_float2(0.5f * (z.y - zc.y), -0.5f * (z.x - zc.x));
    if (m == 0) xH = csub(e, o);  // exp(-i pi) = -1
    v[m] = cadd(e, cmul(o, twz[t + 8 * m]));
  }
}

__device__ __forceinline__ float4 f4(const float2 &a, const float2 &b) {
  return make_float4(a.x, a.y, b.x, b.y);
}

// ZSRC: arrays 0, 1 = d/dx Z, d/dy Z, array 3 = the laplacian (completed by
// the y round trip), array 4 = Z (the z derivative formed here); otherwise
// arrays 0..3 = the four full derivative spectra.
// PLANE: the six GW source spectra are written plane-major, S[kz][x][y]
// (row = x ny + y, element kz rows + row), for the one-pass plane transforms
// (ih_gwplane.cu): each warp stages its four rows in its exchange buffer and
// stores eight kz values x four consecutive y per instruction (32-byte runs;
// the four warps of a CTA complete each 128-byte line of a kz plane).
template <bool ZSRC, bool PLANE>
__global__ void __launch_bounds__(32 * kWarpsW, 4) k_fft_z_rhs_wide(
    const float2 *d4, long long dstride, const float *__restrict__ yfl, const double *ysc,
    float *lap, float *pout, float *rhoout, float2 *s6, long long sstride4, float2 *s6b, int gw,
    double *partials, Geom g, const float2 *__restrict__ twhg, const float2 *__restrict__ twzg) {
  extern __shared__ __align__(16) unsigned char smraw[];
  WideSmem &sm = *reinterpret_cast<WideSmem *>(smraw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int t = lane & 7, grp = lane >> 3, gbase = lane & ~7;
  for (int i = tid; i < kH; i += blockDim.x) sm.twh[i] = twhg[i];
  for (int i = tid; i < 2 * kH; i += blockDim.x) sm.twz[i] = twzg[i];
  __syncthreads();
  const long long rows = (long long)g.nx * g.ny;
  const long long row = ((long long)blockIdx.x * kWarpsW + warp) * kRowsW + grp;
  const bool valid = row < rows;
  float2 *xch = sm.xch[warp][grp];
  const float invnz = (float)(1.0 / (double)g.nz);
  const long long rs = row * (kH + 1);  // first element of the row in a half spectrum

  // fetch row a (x: X_k, xp: X_(H-k)), pre-process, inverse transform
  auto inverse_of = [&](int a, float2 (&v)[16]) {
    float2 x[16], xp[16];
    const float2 *ra = d4 + (ZSRC && a == 2 ? 4 : a) * dstride + rs;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      x[m] = valid ? ra[t + 8 * m] : make_float2(0.f, 0.f);
      xp[m] = valid ? ra[kH - t - 8 * m] : make_float2(0.f, 0.f);
    }
    if (ZSRC && a == 2) {  // i kz Z / nz, zero on the Nyquist index
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const int k = t + 8 * m, kp = kH - k;
        const float f = kfac<float>(g.kzu, k) * invnz;
        const float fp = (kp == kH) ? 0.f : kfac<float>(g.kzu, kp) * invnz;
        x[m] = make_float2(-x[m].y * f, x[m].x * f);
        xp[m] = make_float2(-xp[m].y * fp, xp[m].x * fp);
      }
    }
    zw_c2r_prep(x, xp, t, sm.twz, v);
    zw_inverse(v, t, xch, sm.twh);
  };

  const long long N = g.N;
  const long long e0 = row * (2 * kH) + 4 * t;  // first real of the lane in the row
  // the four inverse transforms in one loop (one copy of the transform code:
  // the kernel's instruction footprint): the laplacian is written out, d/dx
  // and d/dy go to the shared slab, d/dz stays in registers
  float2 dz[16];
#pragma unroll 1
  for (int i = 0; i < 4; ++i) {
    const int a = (i + 3) & 3;  // 3, 0, 1, 2
    float2 v[16];
    inverse_of(a, v);
    if (a == 3) {
      if (valid) {
#pragma unroll
        for (int q = 0; q < 8; ++q)
          *reinterpret_cast<float4 *>(lap + e0 + 32 * q) = f4(v[2 * q], v[2 * q + 1]);
      }
    } else if (a < 2) {
#pragma unroll
      for (int q = 0; q < 8; ++q) sm.grad[warp][a][q][lane] = f4(v[2 * q], v[2 * q + 1]);
    } else {
#pragma unroll
      for (int m = 0; m < 16; ++m) dz[m] = v[m];
    }
  }

  // 4. pointwise energy density and pressure, FP64 partial sums
  const double a_sc = ysc[4];
  const float inv_a2 = (float)(1.0 / (a_sc * a_sc));
  const float m2 = (float)(g.mass * g.mass);
  const float third = (float)(1.0 / 3.0);
  const float phib = (float)ysc[0], pib = (float)ysc[1], psib = (float)ysc[2];
  double dr = 0.0, dp = 0.0;
  if (valid) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const long long e = e0 + 32 * q;
      const float4 ph = *reinterpret_cast<const float4 *>(yfl + e);
      const float4 dph = *reinterpret_cast<const float4 *>(yfl + N + e);
      const float4 ps = *reinterpret_cast<const float4 *>(yfl + 2 * N + e);
      const float4 gx = sm.grad[warp][0][q][lane], gy = sm.grad[warp][1][q][lane];
      const float4 gz = f4(dz[2 * q], dz[2 * q + 1]);
      float4 r4, p4;
      rho_p<float, true>(gx.x, gy.x, gz.x, ph.x, dph.x, ps.x, inv_a2, m2, third, phib, pib, psib,
                         r4.x, p4.x);
      rho_p<float, true>(gx.y, gy.y, gz.y, ph.y, dph.y, ps.y, inv_a2, m2, third, phib, pib, psib,
                         r4.y, p4.y);
      rho_p<float, true>(gx.z, gy.z, gz.z, ph.z, dph.z, ps.z, inv_a2, m2, third, phib, pib, psib,
                         r4.z, p4.z);
      rho_p<float, true>(gx.w, gy.w, gz.w, ph.w, dph.w, ps.w, inv_a2, m2, third, phib, pib, psib,
                         r4.w, p4.w);
      *reinterpret_cast<float4 *>(pout + e) = p4;
      if (rhoout) *reinterpret_cast<float4 *>(rhoout + e) = r4;
      // FP32 over 4 points, FP64 beyond
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
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 gq = f4(dz[2 * q], dz[2 * q + 1]);
      const float4 A = ia < 2 ? sm.grad[warp][ia][q][lane] : gq;
      const float4 Bv = ib < 2 ? sm.grad[warp][ib][q][lane] : gq;
      v[2 * q] = make_float2(A.x * Bv.x, A.y * Bv.y);
      v[2 * q + 1] = make_float2(A.z * Bv.z, A.w * Bv.w);
    }
    zw_forward(v, t, xch, sm.twh);
    float2 xH;
    zw_r2c_post(v, t, gbase, sm.twz, xH);
    if constexpr (PLANE) {
      float2 *arr = pr < 4 ? s6 + pr * sstride4 : s6b + (pr - 4) * sstride4;
#pragma unroll
      for (int m = 0; m < 16; ++m) xch[t + 8 * m] = v[m];
      if (t == 0) xch[kH] = xH;
      __syncwarp();
      const long long row0 = ((long long)blockIdx.x * kWarpsW + warp) * kRowsW;
      const int gs = lane & 3;
      const float2 *xs = sm.xch[warp][gs];
#pragma unroll
      for (int q = 0; q < (kH + 1 + 7) / 8; ++q) {
        const int kz = 8 * q + (lane >> 2);
        if (kz <= kH && row0 + gs < rows) arr[(long long)kz * rows + row0 + gs] = xs[kz];
      }
      __syncwarp();
    } else {
      float2 *dst = (pr < 4 ? s6 + pr * sstride4 : s6b + (pr - 4) * sstride4) + rs;
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
struct WideR2cSmem {
  float2 twh[kH];
  float2 twz[2 * kH];
  float2 xch[kWarpsW][kRowsW][kXch];
};

__global__ void __launch_bounds__(32 * kWarpsW) k_fft_zr2c_wide(const float *__restrict__ in,
                                                               long long istride, float2 *out,
                                                               long long ostride, long long rows,
                                                               const float2 *__restrict__ twhg,
                                                               const float2 *__restrict__ twzg) {
  __shared__ WideR2cSmem sm;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int t = lane & 7, grp = lane >> 3, gbase = lane & ~7;
  for (int i = tid; i < kH; i += blockDim.x) sm.twh[i] = twhg[i];
  for (int i = tid; i < 2 * kH; i += blockDim.x) sm.twz[i] = twzg[i];
  __syncthreads();
  const long long row = ((long long)blockIdx.x * kWarpsW + warp) * kRowsW + grp;
  const bool valid = row < rows;
  const float *src = in + blockIdx.y * istride + row * (2 * kH) + 4 * t;
  float2 v[16];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float4 x = valid ? *reinterpret_cast<const float4 *>(src + 32 * q)
                           : make_float4(0.f, 0.f, 0.f, 0.f);
    v[2 * q] = make_float2(x.x, x.y);
    v[2 * q + 1] = make_float2(x.z, x.w);
  }
  zw_forward(v, t, sm.xch[warp][grp], sm.twh);
  float2 xH;
  zw_r2c_post(v, t, gbase, sm.twz, xH);
  if (valid) {
    float2 *dst = out + blockIdx.y * ostride + row * (kH + 1);
#pragma unroll
    for (int m = 0; m < 16; ++m) dst[t + 8 * m] = v[m];
    if (t == 0) dst[kH] = xH;
  }
}

}  // namespace

bool fused_wide_ok(const Ctx *c) {
  return c->mixed && c->zwide && c->g.h == kH;
}

int zr2c_wide_launch(Ctx *c, const float *in, long long istride, void *out, long long ostride,
                     int count) {
  const Geom &g = c->g;
  const long long rows = (long long)g.nx * g.ny;
  const long long per = (long long)kRowsW * kWarpsW;
  k_fft_zr2c_wide<<<dim3((unsigned)((rows + per - 1) / per), count), 32 * kWarpsW, 0, c->stream>>>(
      in, istride, reinterpret_cast<float2 *>(out), ostride, rows,
      reinterpret_cast<const float2 *>(c->tw_h), reinterpret_cast<const float2 *>(c->tw_z));
  return IH_OK;
}

template <bool ZSRC, bool PLANE>
static void wide_launch_t(Ctx *c, unsigned nblk, size_t sm, const void *d4, long long M,
                          const void *yfl, const double *ysc, void *lap, void *p, void *rho,
                          float2 *s, int gw, double *partials, const Geom &g, const float2 *twh,
                          const float2 *twz) {
  cudaFuncSetAttribute(k_fft_z_rhs_wide<ZSRC, PLANE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sm);
  // row layout: the sources in spectra 0..3, 5, 6 of the RHS block; plane
  // layout: six consecutive spectra of their own buffer
  k_fft_z_rhs_wide<ZSRC, PLANE><<<nblk, 32 * kWarpsW, sm, c->stream>>>(
      (const float2 *)d4, M, (const float *)yfl, ysc, (float *)lap, (float *)p, (float *)rho, s, M,
      s + (PLANE ? 4 : 5) * M, gw, partials, g, twh, twz);
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
  const long long M = g.M;
  const size_t sm = sizeof(WideSmem);
  const float2 *twh = reinterpret_cast<const float2 *>(c->tw_h);
  const float2 *twz = reinterpret_cast<const float2 *>(c->tw_z);
  float2 *s = reinterpret_cast<float2 *>(s6);
  if (zsrc && plane)
    wide_launch_t<true, true>(c, nblk, sm, d4, M, yfl, ysc, lap, p, rho, s, gw, partials, g, twh, twz);
  else if (zsrc)
    wide_launch_t<true, false>(c, nblk, sm, d4, M, yfl, ysc, lap, p, rho, s, gw, partials, g, twh, twz);
  else if (plane)
    wide_launch_t<false, true>(c, nblk, sm, d4, M, yfl, ysc, lap, p, rho, s, gw, partials, g, twh, twz);
  else
    wide_launch_t<false, false>(c, nblk, sm, d4, M, yfl, ysc, lap, p, rho, s, gw, partials, g, twh, twz);
  *nblk_out = (int)nblk;
  return IH_OK;
}

}  // namespace ih
