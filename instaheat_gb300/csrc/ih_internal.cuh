// ih_internal.cuh -- private types and cross-file declarations of
// libinstaheat_gpu.so (GB300, sm_103a).
//
// Device data layout
// ------------------
// A state vector (the reference's `field`, `dfield`, the DOPRI853 stage
// vectors k2..k12, k_tmp, field_new) is split into
//   fl : T[Nf], Nf = 4N + 4Next, segments phi, dphi, psi, dpsi (N each, real
//        space, [x][y][z]) then h1, h2, dh1, dh2 (Next each, interleaved
//        complex half spectrum [x][y][z/2+1]) -- the reference order without a;
//   sc : double[8], sc[0..3] the homogeneous (k = 0) parts of phi, dphi, psi,
//        dpsi and sc[4] the scale factor a.
// The value of component i of segment s < 4 is sc[s] + fl[i]; h and a are
// fl and sc[4] alone.  In the plain FP64 form T = double and sc[0..3] stay 0,
// so fl is exactly the reference's array.  In the mixed form T = float and
// the homogeneous parts live in FP64; the filter pass moves the k = 0 mode of
// fl into sc once per accepted step.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <string>
#include <vector>
#include "../../include/instaheat_gpu.h"

namespace ih {

constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr double kPi = 3.141592653589793238462643383279;
constexpr int kSc = 8;          // doubles of FP64 scalars per vector
constexpr int kMaxPartials = 4096;
constexpr int kDtSlot = 24;     // pinned host slot (doubles into Ctx::hpin) of the try's dt
// Mixed form: each FP32 error-vector element is soft-thresholded by
// eta * eps32 * sum_j |c_j k_j| before it enters the FP64 error norm.
constexpr double kDefaultNoiseEta = 256.0;

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };
template <typename T> using C2 = typename Cplx<T>::type;

// Grid geometry shared by host and device code.
struct Geom {
  int nx, ny, nz, h, mz;        // h = nz/2 (complex z length), mz = nz/2 + 1
  long long N, M, Next, Nf, Ntot;
  double lx, ly, lz;
  double kxu, kyu, kzu;         // 2 pi / L per axis (pars.x.k)
  double kx2, ky2, kz2;         // (2 pi / L)^2 per axis (pars.x.k2)
  double kmax;                  // sqrt(k2_max), setup.c:661-664
  double kxmax, kymax, kzmax;   // filter denominators, setup.c:712-714
  double mass;
  int bins;
  // id / mz for 32-bit ids as (umulhi(id, mz_magic) + id) >> mz_shift
  // (division by an invariant integer, Granlund-Montgomery); ny = 1 << logny
  unsigned mz_magic;
  int mz_shift, logny;
  int pow2;                     // every axis a power of two (else 2^a 3^b: the generic route)
};

// RHS scalars produced on the device by the reduction-finish kernel.
struct RhsScalars {
  double rho_mean, p_mean;      // <rho>, <p> (full values)
  double H, a, a2;              // sqrt(<rho>/3), a, a^2
  double rho_bar, p_bar;        // FP64 homogeneous parts (mixed form)
  double dphi_mean, phi_mean;   // full means (psi solve, constraints)
  double ddphi_mean;            // mean of the dphi-RHS (psi solve)
  int nonfinite;                // set when a reduction saw NaN/Inf
  int pad;
};

struct Vec {                    // one state-shaped vector
  void *fl = nullptr;           // T[Nf]
  double *sc = nullptr;         // double[kSc] (device)
};

// Terms of a DOPRI853/RK4 stage combination (dopri853.c:340-436).
constexpr int kMaxTerms = 12;
// The next stage's input formed by the kernels that write the stage being
// evaluated (k_s): out = base + dt (sum_j coef_j k_j + self k_s), the terms
// in the order of the stand-alone combination (so the result is the same to
// the bit), in place of the RHS input (out is the y the RHS reads: every
// element is read before it is overwritten, by the same thread).
struct NextLin {
  const void *k[kMaxTerms];       // T[Nf] of the earlier stages with a nonzero coefficient
  const double *ksc[kMaxTerms];   // their homogeneous parts
  double coef[kMaxTerms];
  float coeff[kMaxTerms];         // coef rounded to FP32 (the mixed form's fluctuation arithmetic)
  int n;
  double self;                    // the coefficient of k_s (0: none)
  float selff;
  const void *base;               // the step's start state (T[Nf])
  const double *basesc;
  const double *dt;               // the step size (device memory)
  // 1: the position derivatives phi' = dphi, psi' = dpsi, h' = dh (copies of
  // the velocity input) are not written -- stage vectors whose position
  // halves nothing reads (the velocity form); with or without the above
  int skip_pos;
};

// kernel kinds for per-kernel timing and algorithmic-byte accounting
enum KernelKind {
  KK_FFT_XY = 0,        // complex pass along x or y
  KK_FFT_ZR2C,          // real-to-complex pass along z
  KK_FFT_ZC2R,          // complex-to-real pass along z
  KK_X_DERIV4,          // inverse x pass generating the 4 derivative spectra
  KK_XY_RT,             // x or y round trip (derivative spectra of Z)
  KK_X_TENSOR,          // last x pass of the S_ij spectra fused with update_h
  KK_Z_RHS_FUSED,       // last inverse z pass + pointwise + GW products
  KK_UPDATE_H,          // TT projection + tensor equation of motion
  KK_UPDATE_PHI_PSI,    // phi/psi equations of motion
  KK_FILTER,            // spectral filter
  KK_LINCOMB,           // DOPRI853/RK4 stage combination
  KK_DOPRI_FINAL,       // field_new + embedded error sums
  KK_GW_PLANE,          // y and x transforms of the tensor sources, one kz plane per cluster
  KK_UPDATE_H_PLANE,    // update_h reading plane-major tensor sources
  KK_GW_TT_PLANE,       // tensor sources' y/x transforms + TT projection, persistent clusters
  KK_UPDATE_H_TT,       // tensor equation of motion from the projected sources
  KK_COUNT
};
const char *kernel_kind_name(int k);
int kernel_kind_class(int k);     // 0 FFT, 1 pointwise, 2 stepper

struct Timer {                  // per-kind CUDA-event accumulation
  std::vector<cudaEvent_t> ev;  // pairs
  long launches = 0;
  double bytes = 0.0;           // algorithmic bytes of the timed launches
};

// FFT engine variants (fft_autotune picks one per pass)
enum FftVariant {
  FV_STOCKHAM = 0,      // shared-memory Stockham, tile of one 128-byte line of pencils
  FV_TWOSTEP = 1,       // register two-step, tile of one 128-byte line
  FV_TWOSTEP_HALF = 2,  // register two-step, tile of half a line
  FV_PIPELINED = 3,     // register two-step, persistent CTAs, cp.async double buffering
  FV_THREESTEP = 4,     // three register steps of <= 8 values (x/y passes only)
  FV_TWOSTEP_HALF_OCC = 5,  // FV_TWOSTEP_HALF compiled for 7 CTAs per SM (x/y passes, FP32)
  FV_COUNT
};

struct Ctx {
  ih_params p{};
  Geom g{};
  int mixed = 0;                // IH_PREC_MIXED
  size_t tsize = 8;             // sizeof(T)
  cudaStream_t stream = nullptr;
  int num_sms = 0;              // multiprocessors of the device
  std::string err;
  size_t dev_bytes = 0;
  unsigned long long calls_rhs = 0;
  unsigned long long launches = 0;

  // FFT tables (T complex): exp(-2 pi i k / L) for L = nx, ny, h and nz.
  void *tw_x = nullptr, *tw_y = nullptr, *tw_h = nullptr, *tw_z = nullptr;

  // RHS temporaries
  void *spec[7] = {};           // complex M each (T)
  void *rbuf[4] = {};           // real N each: 0 lap, 1 p (fluct), 2 rho (fluct), 3 lap psi
  void *gscratch = nullptr;     // real 6N: derivative fields / GW products of the generic route
  void *mask = nullptr;         // filter mask, M values of T
  double *partials = nullptr;   // partials_cap doubles
  long long partials_cap = 0;
  RhsScalars *rs = nullptr;     // device
  RhsScalars rs_host{};
  // device, 4 * bins + 128 doubles: 4 spectra, then (offsets after 4 * bins)
  // 0-27 constraints + summaries, 28-29 means, 40-42 psi means, 48-50 error
  // sums, 64-67 means of the reference layout, 72-83 error breakdown,
  // 100-101 rms, 112-113 host-array mean / variance
  double *diag = nullptr;
  double *hpin = nullptr;       // pinned host staging: small values
  size_t hpin_bytes = 0;

  // state and stepper vectors
  Vec y, ynew, ytmp, k[13];     // k[1..12] stage RHS, k[1] = dfield
  Vec kd[3], dense;             // dense output: stages 14..16, the interpolated state
  int dense_ready = 0;          // the last accepted DOPRI853 step's stages are intact
  int dense_stages = 0;         // stages 14..16 of that step are evaluated
  int dense_vel = 0;            // that step combined its stages in the velocity form
  int try_vel = 0;              // the form of the last try
  double dense_t0 = 0.0, dense_h = 0.0;  // that step's start and size
  int step_start_valid = 0;     // ynew holds the state at the start of the last step
  double t = 0.0;
  int have_state = 0, dopri_ready = 0;
  ih_dopri_cfg cfg{};
  double dt_next = 0.0, err_old = 1.0e-4;
  int reject = 0;
  long n_ok = 0, n_bad = 0, n_stp = 0, n_tries = 0;
  double last_err = 0.0;

  // host staging for transfers
  void *stage_dev = nullptr;    // FP64 device buffer of Ntot (reference layout)

  // profiling
  int prof_on = 0;
  Timer timers[KK_COUNT];
  cudaEvent_t tev[2] = {nullptr, nullptr};  // ih_timer_start/stop
  double noise_eta = 0.0;       // FP32 rounding floor factor of the error norm
  int err_diag = 0;             // per-segment error-norm breakdown on/off
  // accepted-step history (features of the learned proposer)
  double hist_dt[4] = {0, 0, 0, 0}, hist_err[4] = {0, 0, 0, 0};
  int hist_n = 0;
  ih_mlp *proposer = nullptr;
  float *feat_dev = nullptr;    // 16 floats: 12 features, output at [12]
  double dt_next_pi = 0.0;      // the controller's own proposal of the last step

  // last output flag results available
  int have_output = 0;

  // CUDA graphs of the DOPRI853 try and of the filtered post-step RHS, one per
  // combination of the vectors they touch (see ih_stepper.cu)
  struct Graph {
    int kind = 0;               // 0 try, 1 post-step RHS
    unsigned epoch = 0;
    const void *key[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaGraphExec_t exec = nullptr;
    unsigned long long kernels = 0, rhs_calls = 0;
  };
  std::vector<Graph> graphs;
  unsigned graph_epoch = 0;     // advanced when a captured parameter changes
  int graphs_on = 1;
  double *dt_dev = nullptr;     // step size of the current try (device)

  // FFT engines of the x/y passes (per axis) and of the fused x pass, chosen
  // by fft_autotune; Stockham with 128-byte tiles until tuned
  int xy_var[2] = {0, 0};
  int d4_var = 0;
  int rt_var[2] = {FV_TWOSTEP_HALF, FV_TWOSTEP_HALF};  // x, y round trips (two-step forms)
  int roundtrip = 1;  // RHS without filter/output: round trips instead of full spectra
  int tensor_fused = 0;  // update_h fused into the last x pass (autotuner's choice)
  int gw_plane = 0;      // tensor sources plane-major: 1 one cluster per plane, 2 persistent,
                         // 3 persistent with the projection (k_gw_tt_plane + k_update_h_tt)
  int gw_clusters = 0;   // resident clusters of the persistent plane transforms
  int gw_tt_clusters = 0;  // resident clusters of k_gw_tt_plane
  int *waitflag = nullptr;  // device int: a bounded device-side wait timed out
  void *gwbuf = nullptr;    // plane-major tensor sources: 6 spectra of M complex (T)
  int zwide = 1;         // the wide-row z passes where they apply (nz = 256)
  int gw_slab = 0;       // kz slab width of the tensor sources' y/x passes (0: whole arrays)
  int stage_fusion = 0;  // DOPRI853 stage inputs formed by the RHS of the previous stage
  int velocity_form = 1; // mixed form: stage combinations from the velocity halves only
  int skip_pos = 0;      // set during the stage evaluations of a velocity-form try
  std::string tune_report;
};


// ---------------------------------------------------------------------------
// error helpers
#define IH_CUDA(ctx, call)                                                   \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);       \
      return IH_ERR_CUDA;                                                    \
    }                                                                        \
  } while (0)

#define IH_TRY(expr)                                                         \
  do {                                                                       \
    int s_ = (expr);                                                         \
    if (s_ != IH_OK) return s_;                                              \
  } while (0)

int check_launch(Ctx *c, const char *what);

// profiling brackets around one launch of kernel kind `kind`; `bytes` are
// the launch's algorithmic bytes (each input read once, each output written once)
void prof_begin(Ctx *c, int kind);
void prof_end(Ctx *c, int kind, double bytes);

// ---------------------------------------------------------------------------
// FFT (ih_fft.cu).  All transforms are batched over `count` arrays that are
// `stride` elements apart.  Complex arrays: M = nx*ny*mz elements of C2<T>.
template <typename T>
int fft_r2c(Ctx *c, const T *in, long long in_stride, C2<T> *out,
            long long out_stride, int count);
template <typename T>
int fft_c2r(Ctx *c, C2<T> *in_destroyed, long long in_stride, T *out,
            long long out_stride, int count);
// The three passes, exposed for fused pipelines.
template <typename T>
int fft_zr2c(Ctx *c, const T *in, long long in_stride, C2<T> *out,
             long long out_stride, int count);
template <typename T>
int fft_zc2r(Ctx *c, const C2<T> *in, long long in_stride, T *out,
             long long out_stride, int count);
// axis 0 = x, 1 = y; sign -1 forward, +1 backward; in place.
template <typename T>
int fft_xy(Ctx *c, C2<T> *data, long long stride, int count, int axis,
           int sign);
// forward y then x passes of the six tensor sources (spec arrays 0..3, 5, 6),
// in kz slabs of width w (0: whole arrays)
template <typename T>
int fft_gw_yx(Ctx *c, C2<T> *spec, int w);
// Inverse x-pass that generates the four derivative spectra from phi-hat:
// out[a] = F_a(k) * phihat(k) / N, a = d/dx, d/dy, d/dz, laplacian, then the
// inverse x transform of each; phihat is only read.
template <typename T>
int fft_x_deriv4_inv(Ctx *c, const C2<T> *phihat, C2<T> *out,
                     long long out_stride);
// Round trips along x (axis 0) and y (axis 1) on the z spectra Z of phi:
// d1 = IFFT(i k FFT(Z)) / (L nz), d2 = IFFT(-k^2 FFT(Z)) / (L nz), the
// per-axis derivative spectra of the fused z pass; the y round trip adds its
// d2 and -kz^2 Z / nz to d2 (the x round trip's), completing the laplacian.
template <typename T>
int fft_xy_roundtrip(Ctx *c, const C2<T> *z, C2<T> *d1, C2<T> *d2, int axis);
// The forward x pass of the six S_ij spectra (arrays 0..3 at s03, 4..5 at
// s45, stride M; z and y passes done) fused with update_h: writes the tensor
// segments of out from those of y (toolbox.c:311-346, 363-397).
template <typename T>
int fft_x_tensor(Ctx *c, const C2<T> *s03, const C2<T> *s45, T *y, T *out, double *outsc,
                 const NextLin *next);
// Fused last inverse z pass for the RHS: c2r of the four derivative spectra,
// then per point (grad phi)^2, rho, p (and their FP64 block sums), writes the
// laplacian and p (and rho), and when gw the six products d_i phi d_j phi
// transformed forward along z into six half spectra.  zsrc: the inputs are
// the round-trip outputs (d/dx, d/dy, laplacian, Z in the arrays 0, 1, 3,
// 4), and d/dz comes from Z.
template <typename T>
int fft_z_rhs_fused(Ctx *c, const C2<T> *d4, const T *yfl, const double *ysc,
                    T *lap, T *p, T *rho, C2<T> *s6, int gw, double *partials,
                    int *nblocks_out, int zsrc, int plane = 0);
// The same pass on the wide-row engine (ih_zwide.cu): nz = 256, in the
// context's precision (FP32 mixed form or FP64).
bool fused_wide_ok(const Ctx *c);
// the plain r2c z pass on the wide-row engine (same condition)
int zr2c_wide_launch(Ctx *c, const void *in, long long istride, void *out, long long ostride,
                     int count);
int fused_wide_launch(Ctx *c, const void *d4, const void *yfl, const double *ysc, void *lap,
                      void *p, void *rho, void *s6, int gw, double *partials, int *nblk_out,
                      int zsrc, int plane);
// plane-major tensor sources (ih_gwplane.cu): mixed form, 256^3, wide z pass;
// the six sources live in Ctx::gwbuf (a plane-major write would otherwise
// land in rows of the derivative spectra that other CTAs of the z pass have
// not read yet)
bool gw_plane_ok(const Ctx *c);
int gw_plane_fft(Ctx *c, void *spec, int form);
int update_h_plane(Ctx *c, const void *spec, const void *y, void *out, double *outsc);
int gw_tt_plane(Ctx *c, void *spec);
int update_h_tt(Ctx *c, const void *spec, const void *y, void *out, double *outsc);

int fft_tables(Ctx *c);
// time every engine variant of the x/y passes and the fused x pass on the
// context's scratch spectra and keep the fastest
int fft_autotune(Ctx *c);

// ---------------------------------------------------------------------------
// RHS and helpers (ih_rhs.cu)
// the last forward x pass of the six S_ij spectra + update_h (either form);
// next: also form the tensor segments of the next stage input (in y)
int tensor_last_pass(Ctx *c, void *spec, void *y, void *out, double *outsc,
                     const NextLin *next, bool x_done = false);
int rhs(Ctx *c, double t, Vec &y, Vec &k, int filter, int output,
        const Vec *smry_src, const NextLin *next = nullptr);
int reduce_mean(Ctx *c, const void *arr, long long n, double *dev_out);
int reduce_mean_f64(Ctx *c, const double *arr, long long n, double *dev_out);
// variance of n device doubles around `mean` (toolbox.c:744-754) into
// dev_out[1]; dev_out[0] receives the mean
int variance_f64(Ctx *c, const double *arr, long long n, double mean, double *dev_out);
int ic_fluctuations(Ctx *c, uint64_t seed, double phi0, double dphi0,
                    double a0, double amp, double kcut);
int initial_psi(Ctx *c);
int vec_from_ref(Ctx *c, const double *ref_dev, Vec &v);
int vec_to_ref(Ctx *c, const Vec &v, double *ref_dev);
int vec_copy(Ctx *c, const Vec &src, Vec &dst);
int ifft_any(Ctx *c, const double *in_c_dev, double *out_dev);
int fft_any(Ctx *c, const double *in_dev, double *out_c_dev);
int get_field(Ctx *c, int which, double *dev_out);
int read_output(Ctx *c, ih_output *out);
int mask_init(Ctx *c, void *mask);
int convert_add(Ctx *c, const void *a, double add, long long n, double *out);

// learned proposer (ih_mlp.cu, ih_stepper.cu)
int mlp_forward_async(ih_mlp *m, const float *dx, int n, float *dy, cudaStream_t s);
int step_features(Ctx *c, float *out12);
int field_rms(Ctx *c, const void *arr, long long n, double *dev_out);

// stepper (ih_stepper.cu)
int dopri_init(Ctx *c, const ih_dopri_cfg *cfg, double t0, double dt0, int want_output = 0);
// pieces of perform_step for drivers that interleave several contexts
int try_enqueue(Ctx *c, double dt);
int try_collect(Ctx *c, double *err, double *rho_mean, int *nonfinite);
int try_outcome(Ctx *c, double err, double rho_mean, int nonfinite, double *dt);
int step_accept(Ctx *c, double dt, double err, double rho_mean, int want_output, int tries,
                ih_step_info *info);
int dopri_step(Ctx *c, double dt_try, int want_output, ih_step_info *info);
int rk4_step(Ctx *c, double dt, int want_output);
void dopri_tableau(double *cc, double *a, double *b, double *bhh, double *er);
void dopri_dense_tableau(double *ad, double *d);
int dopri_dense(Ctx *c, double t_out, int want_output);

// launch geometry helper: blocks for n items with `per` items per thread
inline unsigned grid_for(long long n, int threads, int per = 1) {
  long long b = (n + (long long)threads * per - 1) / ((long long)threads * per);
  if (b < 1) b = 1;
  if (b > 152LL * 16) b = 152LL * 16;  // grid-stride beyond 16 CTAs per SM
  return (unsigned)b;
}

}  // namespace ih
