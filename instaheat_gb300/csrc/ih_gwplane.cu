// ih_gwplane.cu -- the tensor sources' y and x transforms in one pass per
// kz plane, and the TT projection + tensor equation of motion reading them
// (mixed form, 256^3).
//
// The six S_ij spectra are written by the fused z pass plane-major,
// S[a][kz][x][y] (each kz plane a contiguous 256 x 256 complex block; the
// six arrays consecutive in their own buffer, Ctx::gwbuf), so
// that one plane's forward y and x transforms can run in one read and one
// write of the plane instead of a y pass and an x pass over whole arrays
// (half the HBM traffic of the row/column engines on these arrays).
//
// k_gw_plane2d: one cluster of 8 CTAs per plane.  CTA r of the cluster
//   1. loads rows x = 32r .. 32r+31 (64 KB, contiguous) with TMA bulk copies
//      (cp.async.bulk, completion on an mbarrier; the wait is bounded and
//      records a timeout in a device flag instead of hanging);
//   2. transforms each row along y: 16 threads per row, n = t + 16m, a
//      16-point DFT over m in registers, the twiddle w256^(t a), an exchange
//      through the row's own shared memory (slots a*16 + (t ^ a): no bank
//      conflicts), a 16-point DFT over t -- thread a ends with y = a + 16b;
//   3. after a cluster barrier (every CTA done with its rows) stores each
//      value into the shared memory of the CTA that owns column y (y / 32)
//      through distributed shared memory, laid out [x][33] (column tiles,
//      padded against bank conflicts); a second cluster barrier publishes
//      the stores;
//   4. transforms its 32 columns along x the same way, in place, and writes
//      them back to the plane (one 256-byte run per x row and warp).
// The exchange reuses the load buffer: after step 2 every thread holds its
// row's values in registers, so the buffer is free once the cluster has
// passed the first barrier.  70 KB of shared memory and 512 threads per CTA:
// two CTAs per SM.
//
// k_update_h_plane: update_h (toolbox.c:311-346, 363-397) over tiles of one
// x row, 32 y and 32 kz: the six sources are read plane-major (256-byte runs
// along y) into shared memory, the state's tensor segments and the outputs
// are read and written in the reference layout (runs along kz); each thread
// then applies the same projection and equation of motion as k_update_h.
//
// k_gw_tt_plane + k_update_h_tt (form 3): the projection moves into the
// plane pass.  Each persistent cluster takes whole kz planes and streams the
// six sources of a plane through its two buffers; after each source's x
// transform every thread adds alpha_a S_a and beta_a S_a of its 16 modes to
// the projected sources n0, n1 it keeps in registers (the projection is
// linear in the S_ij, toolbox.c:363-397).  After the sixth source n0 and n1
// are stored plane-major over the plane's slots of sources 0 and 1 (dead
// once read), so the six sources are read once and never written back;
// k_update_h_tt then applies the equation of motion reading the two
// projected spectra instead of six.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ih_internal.cuh"
#include "ih_fftcore.cuh"
#include "ih_tensor.cuh"

namespace cg = cooperative_groups;

namespace ih {
namespace {

constexpr int kP = 256;                  // plane extent along x and y
constexpr int kCl = 8;                   // CTAs per cluster
constexpr int kRows = kP / kCl;          // rows (and columns) per CTA: 32
constexpr int kLd = kRows + 1;           // padded row length of the column tiles
constexpr int kPlaneThreads = 512;       // 16 threads per row / column
constexpr int kChunkBytes = kRows * kP * 8;   // 64 KB of rows per CTA
constexpr int kCopies = 4;               // bulk copies per chunk (16 KB each)
constexpr long long kWaitLimit = 1LL << 20;   // bounded mbarrier wait (attempts)

struct PlaneSmem {
  float2 buf[kP * kLd];                  // rows [32][256] on load; column tiles [256][33] after
  float2 tw[kP];                         // exp(-2 pi i k/256)
  unsigned long long bar;                // mbarrier of the chunk load
};

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// global -> this CTA's shared memory, completion counted on bar (16-byte
// aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes,
                                          unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// waits for phase `parity` of bar; false after kWaitLimit attempts
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity) {
  for (long long i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// 256-point forward transform of 16 values held by the 16 threads of a line
// (thread t holds v[m] = x[t + 16m]); `line` is the line's 256 slots with
// stride `ld` (complex) between consecutive slots.  On return thread t holds
// v[b] = X[t + 16b].
__device__ __forceinline__ void line_fft256(float2 (&v)[16], int t, float2 *line, int ld,
                                            const float2 *tw) {
  reg_dft<float, 16>(v, tw, 16, -1);
#pragma unroll
  for (int a = 1; a < 16; ++a) v[a] = cmul(v[a], tw[t * a]);
#pragma unroll
  for (int a = 0; a < 16; ++a) line[(a * 16 + (t ^ a)) * ld] = v[a];
  __syncwarp();
#pragma unroll
  for (int s = 0; s < 16; ++s) v[s] = line[(t * 16 + (s ^ t)) * ld];
  __syncwarp();
  reg_dft<float, 16>(v, tw, 16, -1);
}

// One kz plane of one of the six S_ij spectra per cluster: forward y then x
// transforms, in place.  src: the six plane-major spectra, M complex each.
__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kPlaneThreads, 2)
    k_gw_plane2d(float2 *spec, long long M, int mz, const float2 *__restrict__ twg, int *waitflag) {
  extern __shared__ __align__(128) unsigned char smraw[];
  PlaneSmem &sm = *reinterpret_cast<PlaneSmem *>(smraw);
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int tid = threadIdx.x;
  const long long p = blockIdx.x / kCl;          // plane: array a, kz
  const int a = (int)(p / mz), kz = (int)(p % mz);
  float2 *plane = spec + (long long)a * M + (long long)kz * kP * kP;

  if (tid == 0) {
    mbar_init(&sm.bar, 1);
    mbar_expect_tx(&sm.bar, kChunkBytes);
    const char *src = reinterpret_cast<const char *>(plane + (long long)r * kRows * kP);
    char *dst = reinterpret_cast<char *>(sm.buf);
#pragma unroll
    for (int q = 0; q < kCopies; ++q)
      bulk_load(dst + q * (kChunkBytes / kCopies), src + q * (kChunkBytes / kCopies),
                kChunkBytes / kCopies, &sm.bar);
  }
  for (int i = tid; i < kP; i += kPlaneThreads) sm.tw[i] = twg[i];
  __syncthreads();
  const bool loaded = mbar_wait_bounded(&sm.bar, 0);
  if (!loaded) atomicExch(waitflag, 1);  // the results of this plane are then void

  // y transforms of the CTA's 32 rows
  const int t = tid & 15;
  const int row = tid >> 4;
  float2 v[16];
  float2 *line = sm.buf + row * kP;
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = line[t + 16 * m];
  __syncwarp();
  line_fft256(v, t, line, 1, sm.tw);

  cluster.sync();  // every CTA is done with its rows: the buffers take column tiles
  const int x = r * kRows + row;
#pragma unroll
  for (int b = 0; b < 16; ++b) {
    // y = t + 16 b lives in CTA y / 32 = b / 2, column t + 16 (b & 1)
    float2 *dst = cluster.map_shared_rank(sm.buf, b >> 1);
    dst[x * kLd + t + 16 * (b & 1)] = v[b];
  }
  cluster.sync();  // the column tiles are complete

  // x transforms of the CTA's 32 columns (16 threads each), in place
  const int col = tid >> 4;
  float2 *cline = sm.buf + col;
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = cline[(t + 16 * m) * kLd];
  __syncwarp();
  line_fft256(v, t, cline, kLd, sm.tw);
#pragma unroll
  for (int b = 0; b < 16; ++b) cline[(t + 16 * b) * kLd] = v[b];
  __syncthreads();

  // write back: columns 32r .. 32r+31 of every x row
  const int warp = tid >> 5, lane = tid & 31;
  float2 *out = plane + r * kRows + lane;
#pragma unroll 4
  for (int xr = warp; xr < kP; xr += kPlaneThreads / 32)
    out[(long long)xr * kP] = sm.buf[xr * kLd + lane];
  // a CTA whose load timed out waits once more (bounded) for its copies in
  // flight before it exits
  if (!loaded) mbar_wait_bounded(&sm.bar, 0);
}

// Persistent form: each cluster walks planes p = cluster, cluster + clusters,
// ... with two buffers per CTA; while plane i is transformed, the TMA load of
// plane i + 1 is already in flight (issued when plane i - 1's buffer was
// released), so the memory pipe does not idle during the transforms.  One
// CTA per SM (two 67.6 KB buffers); the grid holds exactly the clusters that
// can be resident.  Same arithmetic as k_gw_plane2d.
struct PlaneSmem2 {
  float2 buf[2][kP * kLd];
  float2 tw[kP];
  unsigned long long bar[2];
};

__device__ __forceinline__ void load_chunk(float2 *spec, long long M, int mz, long long p, int r,
                                           float2 *dst, unsigned long long *bar) {
  const int a = (int)(p / mz), kz = (int)(p % mz);
  const float2 *plane = spec + (long long)a * M + (long long)kz * kP * kP;
  const char *src = reinterpret_cast<const char *>(plane + (long long)r * kRows * kP);
  mbar_expect_tx(bar, kChunkBytes);
#pragma unroll
  for (int q = 0; q < kCopies; ++q)
    bulk_load(reinterpret_cast<char *>(dst) + q * (kChunkBytes / kCopies),
              src + q * (kChunkBytes / kCopies), kChunkBytes / kCopies, bar);
}

__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kPlaneThreads, 1)
    k_gw_plane2p(float2 *spec, long long M, int mz, long long nplanes,
                 const float2 *__restrict__ twg, int *waitflag) {
  extern __shared__ __align__(128) unsigned char smraw[];
  PlaneSmem2 &sm = *reinterpret_cast<PlaneSmem2 *>(smraw);
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int tid = threadIdx.x;
  const long long cid = blockIdx.x / kCl, ncl = gridDim.x / kCl;
  if (tid == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    if (cid < nplanes) load_chunk(spec, M, mz, cid, r, sm.buf[0], &sm.bar[0]);
    if (cid + ncl < nplanes) load_chunk(spec, M, mz, cid + ncl, r, sm.buf[1], &sm.bar[1]);
  }
  for (int i = tid; i < kP; i += kPlaneThreads) sm.tw[i] = twg[i];
  __syncthreads();
  const int t = tid & 15, row = tid >> 4, col = tid >> 4;
  const int warp = tid >> 5, lane = tid & 31;
  int it = 0;
  bool late = false;
  for (long long p = cid; p < nplanes; p += ncl, ++it) {
    const int cur = it & 1;
    float2 *buf = sm.buf[cur];
    if (!mbar_wait_bounded(&sm.bar[cur], (unsigned)((it >> 1) & 1))) {
      atomicExch(waitflag, 1);
      late = true;
    }
    // y transforms of the CTA's 32 rows
    float2 v[16];
    float2 *line = buf + row * kP;
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = line[t + 16 * m];
    __syncwarp();
    line_fft256(v, t, line, 1, sm.tw);
    cluster.sync();
    const int x = r * kRows + row;
#pragma unroll
    for (int b = 0; b < 16; ++b) {
      float2 *dst = cluster.map_shared_rank(buf, b >> 1);
      dst[x * kLd + t + 16 * (b & 1)] = v[b];
    }
    cluster.sync();
    // x transforms of the CTA's 32 columns
    float2 *cline = buf + col;
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = cline[(t + 16 * m) * kLd];
    __syncwarp();
    line_fft256(v, t, cline, kLd, sm.tw);
#pragma unroll
    for (int b = 0; b < 16; ++b) cline[(t + 16 * b) * kLd] = v[b];
    __syncthreads();
    const int a = (int)(p / mz), kz = (int)(p % mz);
    float2 *out = spec + (long long)a * M + (long long)kz * kP * kP + r * kRows + lane;
#pragma unroll 4
    for (int xr = warp; xr < kP; xr += kPlaneThreads / 32)
      out[(long long)xr * kP] = buf[xr * kLd + lane];
    __syncthreads();  // every read of buf is done: it takes the plane after next
    if (tid == 0 && p + 2 * ncl < nplanes) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      load_chunk(spec, M, mz, p + 2 * ncl, r, buf, &sm.bar[cur]);
    }
  }
  if (late) {  // as k_gw_tt_plane: the last copy into each buffer
    for (int q = 0; q < 2; ++q) {
      const int last = it - 1 - ((it - 1 - q) & 1);
      if (last >= 0) mbar_wait_bounded(&sm.bar[q], (unsigned)((last >> 1) & 1));
    }
  }
}

// update_h over plane-major sources; tile = one x row, 32 y, up to 32 kz
constexpr int kTileY = 32, kTileK = 32;

struct UhSmem {
  float2 s[6][kTileK][kTileY + 1];
};

__global__ void __launch_bounds__(256, 3)
    k_update_h_plane(const float2 *__restrict__ spec, const float *__restrict__ y,
                     float *__restrict__ out, const RhsScalars *rs, Geom g, int skip_pos,
                     double *outsc) {
  extern __shared__ __align__(16) unsigned char uhraw[];
  UhSmem &sm = *reinterpret_cast<UhSmem *>(uhraw);
  const int x = blockIdx.x;
  const int y0 = blockIdx.y * kTileY;
  const int k0 = blockIdx.z * kTileK;
  const int nk = min(kTileK, g.mz - k0);
  const long long M = g.M;
  const long long plane = (long long)g.nx * g.ny;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // the six sources: one 256-byte run along y per (array, kz)
  for (int q = warp; q < 6 * nk; q += 8) {
    const int a = q / nk, kl = q - a * nk;
    const long long base = (long long)a * M + (long long)(k0 + kl) * plane +
                           (long long)x * g.ny + y0;
    sm.s[a][kl][lane] = spec[base + lane];
  }
  __syncthreads();
  const TensorConsts<float> tc(rs);
  float mx = 0.f;
  const int kl = lane;
  if (kl < nk) {
    const int kz = k0 + kl;
    // the state's tensor entries of the thread's four modes, loaded before
    // any arithmetic so that all sixteen loads are in flight together
    HVals<float> hq[kTileY / 8];
#pragma unroll
    for (int q = 0; q < kTileY / 8; ++q)
      tensor_load<float>(g, ((long long)x * g.ny + y0 + warp + 8 * q) * g.mz + kz, y, hq[q]);
#pragma unroll
    for (int q = 0; q < kTileY / 8; ++q) {
      const int yl = warp + 8 * q;
      const int j = y0 + yl;
      const long long id = ((long long)x * g.ny + j) * g.mz + kz;
      Mode m;
      m.i = x;
      m.j = j;
      m.k = kz;
      C2<float> n0 = mk2c<float>(0.f, 0.f), n1 = mk2c<float>(0.f, 0.f);
      float ksq = 0.f;
      if (id != 0) {  // the zero mode has no sources
        const C2<float> v[6] = {sm.s[0][kl][yl], sm.s[1][kl][yl], sm.s[2][kl][yl],
                                sm.s[3][kl][yl], sm.s[4][kl][yl], sm.s[5][kl][yl]};
        const ModeK<float> qk = mode_k<float>(g, m);
        ksq = qk.ksq;
        tensor_sources<float>(m, qk, v, n0, n1);
      }
      C2<float> o3, o4;
      tensor_eom_core<float>(g, id, n0, n1, ksq, tc, hq[q], out, skip_pos, o3, o4);
      mx = fmaxf(mx, fmaxf(fmaxf(fabsf(o3.x), fabsf(o3.y)), fmaxf(fabsf(o4.x), fabsf(o4.y))));
    }
  }
  dh_max_store<float>(mx, outsc);
}

// n0 += alpha_a S_a, n1 += beta_a S_a over the 16 modes x = t + 16 b of
// column y = yj of plane kz (v[b] = S_a there)
__device__ __forceinline__ void tt_accumulate(const Geom &g, int a, int t, int ja, float ky, int kz,
                                              int yj, const float2 (&v)[16], float2 (&n0)[16],
                                              float2 (&n1)[16]) {
  const float kzf = (float)g.kzu * (float)kz;
  const float kzz = (float)g.kz2 * (float)kz * (float)kz;
  const float kyy = (float)g.ky2 * (float)ja * (float)ja;
  const int branch = kz != 0 ? 0 : (yj != 0 ? 1 : 2);
#pragma unroll
  for (int b = 0; b < 16; ++b) {
    const int xi = t + 16 * b;
    const int ia = xi > kP / 2 ? kP - xi : xi;
    const float kx = (float)g.kxu * (float)(xi > kP / 2 ? xi - kP : xi);
    float ksq = kzz;
    ksq += (float)g.kx2 * (float)ia * (float)ia;
    ksq += kyy;
    const float inv = ksq > 0.f ? 1.f / ksq : 0.f;
    float al, be;
    tensor_coef<float>(a, branch, kx, ky, kzf, kx * inv, ky * inv, kzf * inv, al, be);
    n0[b].x += al * v[b].x;
    n0[b].y += al * v[b].y;
    n1[b].x += be * v[b].x;
    n1[b].y += be * v[b].y;
  }
}

// Form 3, pass 1: y and x transforms of the six sources of each kz plane
// and their TT projection.  Cluster c takes planes kz = c, c + C, ... (C
// resident clusters); its iteration it handles source a = it % 6 of plane
// kz = c + (it / 6) C, in buffer it % 2, with the load of iteration it + 2
// issued as soon as the buffer is free.  Thread (column j = tid / 16, t =
// tid % 16) of CTA r ends each x transform with the modes x = t + 16 b,
// y = 32 r + j, b = 0..15, and keeps n0, n1 of those 16 modes in registers
// across the six sources.
__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kPlaneThreads, 1)
    k_gw_tt_plane(float2 *spec, Geom g, const float2 *__restrict__ twg, int *waitflag) {
  extern __shared__ __align__(128) unsigned char smraw[];
  PlaneSmem2 &sm = *reinterpret_cast<PlaneSmem2 *>(smraw);
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int tid = threadIdx.x;
  const int mz = g.mz;
  const long long M = g.M;
  const int cid = (int)(blockIdx.x / kCl), ncl = (int)(gridDim.x / kCl);
  const int nloc = cid < mz ? (mz - 1 - cid) / ncl + 1 : 0;  // planes of this cluster
  const int nit = 6 * nloc;
  if (tid == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    for (int q = 0; q < 2 && q < nit; ++q)
      load_chunk(spec, M, mz, (long long)q * mz + cid, r, sm.buf[q], &sm.bar[q]);
  }
  for (int i = tid; i < kP; i += kPlaneThreads) sm.tw[i] = twg[i];
  __syncthreads();
  const int t = tid & 15, row = tid >> 4;  // y pass: row x = 32 r + row; x pass: column y
  const int warp = tid >> 5, lane = tid & 31;
  const int yj = r * kRows + row;
  const int ja = yj > kP / 2 ? kP - yj : yj;
  const float ky = (float)g.kyu * (float)(yj > kP / 2 ? yj - kP : yj);
  float2 n0[16], n1[16];
  bool late = false;  // a wait gave up: the results are void (waitflag set)
  for (int it = 0; it < nit; ++it) {
    const int cur = it & 1, a = it % 6;
    const int kz = cid + (it / 6) * ncl;
    float2 *buf = sm.buf[cur];
    if (a == 0) {
#pragma unroll
      for (int b = 0; b < 16; ++b) n0[b] = n1[b] = make_float2(0.f, 0.f);
    }
    if (!mbar_wait_bounded(&sm.bar[cur], (unsigned)((it >> 1) & 1))) {
      atomicExch(waitflag, 1);
      late = true;
    }
    // y transforms of the CTA's 32 rows
    float2 v[16];
    float2 *line = buf + row * kP;
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = line[t + 16 * m];
    __syncwarp();
    line_fft256(v, t, line, 1, sm.tw);
    cluster.sync();  // every CTA is done with its rows: the buffers take column tiles
    const int x = r * kRows + row;
#pragma unroll
    for (int b = 0; b < 16; ++b) {
      float2 *dst = cluster.map_shared_rank(buf, b >> 1);
      dst[x * kLd + t + 16 * (b & 1)] = v[b];
    }
    cluster.sync();  // the column tiles are complete
    // x transforms of the CTA's 32 columns
    float2 *cline = buf + row;
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = cline[(t + 16 * m) * kLd];
    __syncwarp();
    line_fft256(v, t, cline, kLd, sm.tw);
    __syncthreads();  // every read of buf is done
    if (a < 5 && tid == 0 && it + 2 < nit) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      const int i2 = it + 2;
      load_chunk(spec, M, mz, (long long)(i2 % 6) * mz + cid + (i2 / 6) * ncl, r, buf,
                 &sm.bar[cur]);
    }
    // the projection of source a (coefficients as k_fft_x_tensor, FP32)
    tt_accumulate(g, a, t, ja, ky, kz, yj, v, n0, n1);
    if (a == 5) {
      // n0 then n1, transposed through buf (free: its next load is not yet
      // issued), over the plane's slots of sources 0 and 1: rows of 32 y
      const bool zero_mode = kz == 0 && yj == 0 && t == 0;  // x = y = kz = 0: no sources
#pragma unroll
      for (int s = 0; s < 2; ++s) {
#pragma unroll
        for (int b = 0; b < 16; ++b) {
          float2 w = s == 0 ? n0[b] : n1[b];
          if (b == 0 && zero_mode) w = make_float2(0.f, 0.f);
          buf[(t + 16 * b) * kLd + row] = w;
        }
        __syncthreads();
        float2 *o = spec + (long long)s * M + (long long)kz * kP * kP + r * kRows + lane;
#pragma unroll 4
        for (int xr = warp; xr < kP; xr += kPlaneThreads / 32)
          o[(long long)xr * kP] = buf[xr * kLd + lane];
        __syncthreads();
      }
      if (tid == 0 && it + 2 < nit) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const int i2 = it + 2;
        load_chunk(spec, M, mz, (long long)(i2 % 6) * mz + cid + (i2 / 6) * ncl, r, buf,
                   &sm.bar[cur]);
      }
    }
  }
  // after a wait that gave up, wait (bounded) once more for the last copy
  // into each buffer before the CTA's shared memory is released
  if (late) {
    for (int q = 0; q < 2; ++q) {
      const int last = nit - 1 - ((nit - 1 - q) & 1);
      if (last >= 0) mbar_wait_bounded(&sm.bar[q], (unsigned)((last >> 1) & 1));
    }
  }
}

// Form 3, pass 2: the equation of motion from the projected sources n0, n1
// (plane-major, sources 0 and 1 of spec) over tiles of one x row, 32 y and
// 32 kz, as k_update_h_plane without the projection.
struct UhTtSmem {
  float2 s[2][kTileK][kTileY + 1];
};

__global__ void __launch_bounds__(256, 4)
    k_update_h_tt(const float2 *__restrict__ spec, const float *__restrict__ y,
                  float *__restrict__ out, const RhsScalars *rs, Geom g, int skip_pos,
                  double *outsc) {
  __shared__ UhTtSmem sm;
  const int x = blockIdx.x;
  const int y0 = blockIdx.y * kTileY;
  const int k0 = blockIdx.z * kTileK;
  const int nk = min(kTileK, g.mz - k0);
  const long long M = g.M;
  const long long plane = (long long)g.nx * g.ny;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int q = warp; q < 2 * nk; q += 8) {
    const int a = q / nk, kl = q - a * nk;
    sm.s[a][kl][lane] =
        spec[(long long)a * M + (long long)(k0 + kl) * plane + (long long)x * g.ny + y0 + lane];
  }
  __syncthreads();
  const TensorConsts<float> tc(rs);
  float mx = 0.f;
  const int kl = lane;
  if (kl < nk) {
    const int kz = k0 + kl;
    HVals<float> hq[kTileY / 8];
#pragma unroll
    for (int q = 0; q < kTileY / 8; ++q)
      tensor_load<float>(g, ((long long)x * g.ny + y0 + warp + 8 * q) * g.mz + kz, y, hq[q]);
#pragma unroll
    for (int q = 0; q < kTileY / 8; ++q) {
      const int yl = warp + 8 * q;
      const long long id = ((long long)x * g.ny + y0 + yl) * g.mz + kz;
      Mode m;
      m.i = x;
      m.j = y0 + yl;
      m.k = kz;
      const float ksq = id != 0 ? mode_k<float>(g, m).ksq : 0.f;
      C2<float> o3, o4;
      tensor_eom_core<float>(g, id, sm.s[0][kl][yl], sm.s[1][kl][yl], ksq, tc, hq[q], out,
                             skip_pos, o3, o4);
      mx = fmaxf(mx, fmaxf(fmaxf(fabsf(o3.x), fabsf(o3.y)), fmaxf(fabsf(o4.x), fabsf(o4.y))));
    }
  }
  dh_max_store<float>(mx, outsc);
}

}  // namespace

bool gw_plane_ok(const Ctx *c) {
  return c->mixed && fused_wide_ok(c) && c->g.nx == kP && c->g.ny == kP && c->p.enable_gw &&
         c->waitflag != nullptr && c->gwbuf != nullptr;
}

// form 1: one cluster per plane; form 2: persistent clusters with the next
// plane's load in flight
int gw_plane_fft(Ctx *c, void *spec, int form) {
  const Geom &g = c->g;
  const long long nplanes = 6LL * g.mz;
  prof_begin(c, KK_GW_PLANE);
  if (form == 2) {
    const size_t smem = sizeof(PlaneSmem2);
    IH_CUDA(c, cudaFuncSetAttribute(k_gw_plane2p, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
    if (c->gw_clusters <= 0) {
      // the clusters that can be resident at once: the persistent grid
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(kCl * 64, 1, 1);
      cfg.blockDim = dim3(kPlaneThreads, 1, 1);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = c->stream;
      int ncl = 0;
      IH_CUDA(c, cudaOccupancyMaxActiveClusters(&ncl, (const void *)k_gw_plane2p, &cfg));
      if (ncl < 1) {
        c->err = "no cluster of 8 CTAs fits the device";
        return IH_ERR_CUDA;
      }
      c->gw_clusters = ncl;
    }
    const long long ncl = c->gw_clusters < nplanes ? c->gw_clusters : nplanes;
    k_gw_plane2p<<<(unsigned)(ncl * kCl), kPlaneThreads, smem, c->stream>>>(
        reinterpret_cast<float2 *>(spec), g.M, g.mz, nplanes,
        reinterpret_cast<const float2 *>(c->tw_z), c->waitflag);
  } else {
    const size_t smem = sizeof(PlaneSmem);
    static_assert(sizeof(PlaneSmem) <= 113 * 1024, "two CTAs per SM");
    IH_CUDA(c, cudaFuncSetAttribute(k_gw_plane2d, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
    k_gw_plane2d<<<(unsigned)(nplanes * kCl), kPlaneThreads, smem, c->stream>>>(
        reinterpret_cast<float2 *>(spec), g.M, g.mz, reinterpret_cast<const float2 *>(c->tw_z),
        c->waitflag);
  }
  prof_end(c, KK_GW_PLANE, 12.0 * g.M * sizeof(float2));
  return check_launch(c, form == 2 ? "k_gw_plane2p" : "k_gw_plane2d");
}

int update_h_plane(Ctx *c, const void *spec, const void *y, void *out, double *outsc) {
  const Geom &g = c->g;
  dim3 grid((unsigned)g.nx, (unsigned)(g.ny / kTileY), (unsigned)((g.mz + kTileK - 1) / kTileK));
  const size_t smem = sizeof(UhSmem);
  IH_CUDA(c, cudaFuncSetAttribute(k_update_h_plane, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  prof_begin(c, KK_UPDATE_H_PLANE);
  k_update_h_plane<<<grid, 256, smem, c->stream>>>(
      reinterpret_cast<const float2 *>(spec), reinterpret_cast<const float *>(y),
      reinterpret_cast<float *>(out), c->rs, g, c->skip_pos, outsc);
  prof_end(c, KK_UPDATE_H_PLANE,
           6.0 * g.M * sizeof(float2) + (c->skip_pos ? 6.0 : 8.0) * g.Next * sizeof(float));
  return check_launch(c, "k_update_h_plane");
}

// the clusters of 8 that can be resident at once (the persistent grid)
static int resident_clusters(const void *kernel, size_t smem, cudaStream_t s, int *ncl) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kCl * 64, 1, 1);
  cfg.blockDim = dim3(kPlaneThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  *ncl = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(ncl, kernel, &cfg);
  return e == cudaSuccess && *ncl >= 1 ? IH_OK : IH_ERR_CUDA;
}

int gw_tt_plane(Ctx *c, void *spec) {
  const Geom &g = c->g;
  const size_t smem = sizeof(PlaneSmem2);
  IH_CUDA(c, cudaFuncSetAttribute(k_gw_tt_plane, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  if (c->gw_tt_clusters <= 0) {
    int ncl = 0;
    if (resident_clusters((const void *)k_gw_tt_plane, smem, c->stream, &ncl) != IH_OK) {
      c->err = "no cluster of 8 CTAs of k_gw_tt_plane fits the device";
      return IH_ERR_CUDA;
    }
    c->gw_tt_clusters = ncl;
  }
  const int ncl = c->gw_tt_clusters < g.mz ? c->gw_tt_clusters : g.mz;
  prof_begin(c, KK_GW_TT_PLANE);
  k_gw_tt_plane<<<(unsigned)(ncl * kCl), kPlaneThreads, smem, c->stream>>>(
      reinterpret_cast<float2 *>(spec), g, reinterpret_cast<const float2 *>(c->tw_z), c->waitflag);
  prof_end(c, KK_GW_TT_PLANE, 8.0 * g.M * sizeof(float2));
  return check_launch(c, "k_gw_tt_plane");
}

int update_h_tt(Ctx *c, const void *spec, const void *y, void *out, double *outsc) {
  const Geom &g = c->g;
  dim3 grid((unsigned)g.nx, (unsigned)(g.ny / kTileY), (unsigned)((g.mz + kTileK - 1) / kTileK));
  prof_begin(c, KK_UPDATE_H_TT);
  k_update_h_tt<<<grid, 256, 0, c->stream>>>(reinterpret_cast<const float2 *>(spec),
                                             reinterpret_cast<const float *>(y),
                                             reinterpret_cast<float *>(out), c->rs, g, c->skip_pos,
                                             outsc);
  prof_end(c, KK_UPDATE_H_TT,
           2.0 * g.M * sizeof(float2) + (c->skip_pos ? 6.0 : 8.0) * g.Next * sizeof(float));
  return check_launch(c, "k_update_h_tt");
}

}  // namespace ih

// ---------------------------------------------------------------------------
// measurement: the plane transforms alone on a buffer of their own (six
// spectra of 256 x 256 x mz complex FP32, mz = 129 for 256^3: 405 MB, larger
// than L2), for CUDA-event timing and small-case profiling.  No reference
// counterpart.
extern "C" int ih_gw_plane_probe(int device, int form, int mz, int reps, double *ms_per_launch) {
  using namespace ih;
  if (!ms_per_launch || reps < 1 || mz < 1 || form < 1 || form > 3) return IH_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return IH_ERR_CUDA;
  const long long M = (long long)kP * kP * mz, nplanes = 6LL * mz;
  float2 *buf = nullptr, *tw = nullptr;
  int *flag = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = IH_ERR_CUDA;
  float ms = 0.f;
  int ncl = 0;
  float2 htw[kP];
  // k vectors of a 256 x 256 x 2(mz - 1) grid in a box of 20 (form 3's
  // projection; they change the arithmetic, not the memory traffic)
  Geom g = {};
  g.nx = g.ny = kP;
  g.nz = 2 * (mz - 1);
  g.h = mz - 1;
  g.mz = mz;
  g.M = M;
  g.kxu = g.kyu = g.kzu = kTwoPi / 20.0;
  g.kx2 = g.ky2 = g.kz2 = g.kxu * g.kxu;
  for (int k = 0; k < kP; ++k) {
    const double ang = 6.283185307179586476925286766559 * k / kP;
    htw[k] = make_float2((float)cos(ang), (float)-sin(ang));
  }
  if (cudaMalloc(&buf, sizeof(float2) * 6 * M) != cudaSuccess) return IH_ERR_ALLOC;
  if (cudaMalloc(&tw, sizeof htw) != cudaSuccess || cudaMalloc(&flag, sizeof(int)) != cudaSuccess)
    goto done;
  if (cudaMemset(buf, 0, sizeof(float2) * 6 * M) != cudaSuccess ||
      cudaMemset(flag, 0, sizeof(int)) != cudaSuccess ||
      cudaMemcpy(tw, htw, sizeof htw, cudaMemcpyHostToDevice) != cudaSuccess)
    goto done;
  if (cudaFuncSetAttribute(k_gw_plane2d, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(PlaneSmem)) != cudaSuccess ||
      cudaFuncSetAttribute(k_gw_plane2p, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(PlaneSmem2)) != cudaSuccess ||
      cudaFuncSetAttribute(k_gw_tt_plane, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(PlaneSmem2)) != cudaSuccess)
    goto done;
  if (form >= 2) {
    if (resident_clusters(form == 2 ? (const void *)k_gw_plane2p : (const void *)k_gw_tt_plane,
                          sizeof(PlaneSmem2), 0, &ncl) != IH_OK)
      goto done;
    const long long units = form == 2 ? nplanes : mz;
    if (ncl > units) ncl = (int)units;
  }
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) goto done;
  for (int r = 0; r <= reps; ++r) {  // r = 0: warm-up
    if (r == 1) cudaEventRecord(e0);
    if (form == 3)
      k_gw_tt_plane<<<(unsigned)(ncl * kCl), kPlaneThreads, sizeof(PlaneSmem2)>>>(buf, g, tw, flag);
    else if (form == 2)
      k_gw_plane2p<<<(unsigned)(ncl * kCl), kPlaneThreads, sizeof(PlaneSmem2)>>>(buf, M, mz, nplanes,
                                                                                tw, flag);
    else
      k_gw_plane2d<<<(unsigned)(nplanes * kCl), kPlaneThreads, sizeof(PlaneSmem)>>>(buf, M, mz, tw,
                                                                                   flag);
    if (cudaGetLastError() != cudaSuccess) goto done;
  }
  cudaEventRecord(e1);
  if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
    goto done;
  *ms_per_launch = ms / reps;
  st = IH_OK;
done:
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(buf);
  cudaFree(tw);
  cudaFree(flag);
  return st;
}
