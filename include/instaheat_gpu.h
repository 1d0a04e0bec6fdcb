/*
 * instaheat_gpu.h -- C ABI of libinstaheat_gpu.so, the GB300 (sm_103a)
 * implementation of InstaHeat's right-hand side and time steppers.
 *
 * Every entry point takes plain pointers and sizes, returns an int status
 * (IH_OK = 0, see ih_status_string) instead of calling exit(), and is called
 * from one host thread per context.  One context owns one grid on one GPU:
 * its device-resident state, the DOPRI853/RK4 work vectors, the k grids, the
 * filter mask and the FFT tables.
 *
 * State layout (host side, identical to the reference, src/main_template.h:
 * 223-233): f[Ntot], Ntot = 4N + 4Next + 1: phi, dphi, psi, dpsi (N doubles
 * each, row-major [x][y][z]), h1, h2, dh1, dh2 (Next = 2M doubles each, M
 * interleaved complex, r2c half spectrum [x][y][z/2+1]), then a.
 *
 * Precision forms:
 *   IH_PREC_F64   -- plain FP64 everywhere (the reference's arithmetic).
 *   IH_PREC_MIXED -- FP32 fluctuation fields, FFTs and pointwise arithmetic;
 *                    FP64 homogeneous (k = 0) parts of phi, dphi, psi, dpsi,
 *                    FP64 scale factor a, Hubble rate, <rho>, <p>, all
 *                    reductions and the DOPRI853 error norm.
 *
 * The drop-in symbols that the reference's own C code calls (mk_rhs,
 * run_dopri853, run_rk4, fft, ifft, mean, variance, evo_flags) are provided by
 * the C99 host layer declared in instaheat_dropin.h, on top of this ABI.
 */
#ifndef INSTAHEAT_GPU_H
#define INSTAHEAT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    IH_OK = 0,
    IH_ERR_ARG = 1,        /* invalid argument or unsupported grid */
    IH_ERR_CUDA = 2,       /* a CUDA call failed (message in ih_last_error) */
    IH_ERR_ALLOC = 3,      /* device or host allocation failed */
    IH_ERR_STATE = 4,      /* call out of order (e.g. step before init) */
    IH_ERR_UNDERFLOW = 5,  /* DOPRI853 step-size underflow (dopri853.c:280-283) */
    IH_ERR_NAN = 6,        /* non-finite value in a reduction (NaN/Inf flag) */
    IH_ERR_TOO_LARGE = 7   /* input larger than a fixed-size entry point accepts */
};

enum { IH_PREC_F64 = 0, IH_PREC_MIXED = 1 };

/* Grid and physics parameters: the parameters.sh keys of the hot path. */
typedef struct {
    int nx, ny, nz;        /* GRIDPOINTS_X/Y/Z: 2^a 3^b (a >= 1; powers of two take
                              the tuned engines, a factor 3 the mixed-radix route),
                              nx >= ny >= nz >= 8, nx <= 512 */
    double lx, ly, lz;     /* SPATIAL_UPPER_BOUND_* - SPATIAL_LOWER_BOUND_* */
    double mass;           /* MASS (V = m^2 phi^2 / 2) */
    int enable_gw;         /* ENABLE_GW */
    int enable_filter;     /* ENABLE_FFT_FILTER */
    int bins;              /* POWER_SPECTRUM_BINS (field and GW spectra) */
    int precision;         /* IH_PREC_F64 or IH_PREC_MIXED */
    int device;            /* CUDA device ordinal */
} ih_params;

/* DOPRI853 controller parameters (parameters.sh: RELATIVE_TOLERANCE,
 * ABSOLUTE_TOLERANCE, BETA, SAFE, SMALLEST_SCALING, LARGEST_SCALING,
 * MAX_DT_HUBBLE_FRACTION (<= 0 disables the cap), MINIMAL_DELTA_T, MAX_STEPS). */
typedef struct {
    double rtol, atol, beta, safe, minscale, maxscale;
    double max_dt_hubble_fraction, dt_min, max_steps;
} ih_dopri_cfg;

/* Diagnostics of the last RHS evaluated with the output flag
 * (toolbox.c:251-270).  Arrays are caller-owned, `bins` doubles each; any
 * pointer may be NULL. */
typedef struct {
    double *phi_ps, *psi_ps, *rho_ps, *gw;
    double cstr[4];        /* <ham^2>, max|ham|, <mom^2>, max|mom| */
    double smry[6][4];     /* phi, dphi, psi, dpsi, rho, p: mean, var, min, max */
} ih_output;

/* Result of one DOPRI853 perform_step (dopri853.c:271-311). */
typedef struct {
    double t;              /* time after the step */
    double dt_did;         /* accepted step size */
    double dt_next;        /* proposed next step size */
    double err;            /* error() of the accepted try */
    int tries;             /* try_step calls, rejected ones included */
    int status;            /* IH_OK or IH_ERR_UNDERFLOW */
} ih_step_info;

const char *ih_status_string(int status);

/* Sizes N, M, Next, Ntot of a grid (setup.c:228-271, 3D). */
int ih_sizes(int nx, int ny, int nz, size_t *N, size_t *M, size_t *Next,
             size_t *Ntot);

typedef struct ih_context ih_context;

/* Create a context (allocates all device memory for the grid; replaces
 * allocate_external, setup.c:354-477, mk_k_grid 609-666, mk_filter_mask
 * 710-754 and the FFTW plans 524-554). */
int ih_create(const ih_params *p, ih_context **out);
void ih_destroy(ih_context *c);
const char *ih_last_error(const ih_context *c);
/* Device bytes the context holds. */
size_t ih_device_bytes(const ih_context *c);

/* ---- state transfer (host FP64, reference layout) ---- */
/* Upload `field` and set the time.  The DOPRI853 controller state is kept;
 * ih_dopri853_step uses the dfield on the device, so a caller that replaces
 * the state either uploads the matching dfield with ih_set_dstate or calls
 * ih_dopri853_init (which recomputes it with the filtered RHS). */
int ih_set_state(ih_context *c, const double *f_host, double t);
int ih_get_state(ih_context *c, double *f_host);
/* dfield: the RHS of the current state (valid after ih_dopri853_init/step). */
int ih_set_dstate(ih_context *c, const double *df_host);
int ih_get_dstate(ih_context *c, double *df_host);
double ih_time(const ih_context *c);

/* ---- the RHS (toolbox.c:75-88) ---- */
/* mk_rhs on host buffers: uploads f, evaluates, downloads result.  With
 * filter=1 (and ENABLE_FFT_FILTER) f is overwritten by its filtered version,
 * as the reference does (toolbox.c:164-171).  With output=1 the diagnostics
 * are computed and kept for ih_get_output. */
int ih_mk_rhs_host(ih_context *c, double t, double *f, double *result,
                   int filter, int output);
/* mk_rhs on device pointers in the reference layout (FP64, Ntot doubles).
 * f_dev is overwritten when filter=1.  Plain FP64 contexts only. */
int ih_mk_rhs_dev(ih_context *c, double t, double *f_dev, double *result_dev,
                  int filter, int output);
/* <rho>, <p> of the last RHS (the reference's rho_mean, pressure_mean). */
int ih_get_means(const ih_context *c, double *rho_mean, double *pressure_mean);
/* Copy a per-point field of the last RHS to host (N doubles):
 * which = 0 rho, 1 pressure, 2 laplacian of phi (3, the squared gradient, is
 * not kept by the fused RHS pass and returns IH_ERR_ARG). */
int ih_get_field(ih_context *c, int which, double *out_host);
int ih_get_output(ih_context *c, ih_output *out);
/* prepare_and_save_timeslice without save() (toolbox.c:96-104): the RHS of
 * the device state with filter = output = 1; dfield is updated, the state is
 * filtered in place, the diagnostics are kept for ih_get_output. */
int ih_prepare_output(ih_context *c);
unsigned long long ih_calls_rhs(const ih_context *c);

/* mean (toolbox.c:726-734) of n doubles in device memory, FP64 two-stage
 * reduction on the context stream (scratch: the context's partial-sum
 * buffer).  *out_dev is device memory; the call returns once it is written. */
int ih_mean_dev(ih_context *c, const double *f_dev, size_t n, double *out_dev);

/* The same mean without allocating anything, for callers that cannot call
 * cudaMalloc where they need it (a host program that gives all device memory
 * to its own arena up front, a loop that must not pay or risk an allocation,
 * code without an ih_context).  No counterpart in the reference.
 * Scratch is a fixed 32 KiB array inside the library (held on every GPU that
 * loads it until the process exits); it is shared by all calls, so calls that
 * overlap on the GPU race and must be serialised by the caller.  The call
 * runs on the calling thread's current CUDA device and uses that device's
 * copy of the array: f_dev, out_dev and stream must all belong to it (unlike
 * ih_mean_dev, which is tied to its context's device).  Each call looks the
 * array's device address up in the current context; the first call in a
 * context may load the library's kernels there, so make it before any
 * stream capture.  n is limited to ih_mean_dev_noalloc_max_n() = 2^28
 * doubles; larger n returns IH_ERR_TOO_LARGE without launching anything.
 * Runs on `stream` (a cudaStream_t; NULL = the legacy default stream) and
 * returns without waiting; *out_dev is device memory.  On IH_ERR_CUDA the
 * CUDA error is left pending for the caller's cudaGetLastError (a pending
 * error from the caller's earlier work also yields IH_ERR_CUDA). */
int ih_mean_dev_noalloc(const double *f_dev, size_t n, double *out_dev, void *stream);
size_t ih_mean_dev_noalloc_max_n(void);

/* mean and variance (toolbox.c:726-734, 744-754) of n doubles in HOST memory,
 * computed on the device (copied into the context's staging buffer, FP64 block
 * sums): variance = (sum (f-mean)^2 - (sum (f-mean))^2 / n) / (n - 1) around
 * the caller's mean, as the reference computes it.  n <= Ntot of the grid
 * (IH_ERR_TOO_LARGE otherwise). */
int ih_mean_host(ih_context *c, const double *f_host, size_t n, double *out);
int ih_variance_host(ih_context *c, double mean, const double *f_host, size_t n,
                     double *out);

/* ---- FFT autotuner (no reference counterpart; FFTW's planner flag
 * FFTW_DEFAULT_FLAG, parameters.sh, plays this role there) ----
 * Times every engine variant of the x and y passes, of the fused inverse x
 * pass, of the x and y derivative round trips, of the last tensor x pass and
 * the kz slab widths of the tensor sources' y/x passes and, where it
 * applies, the plane-major tail of the tensor sources (pass 8 below) of the
 * RHS on the context's scratch spectra and keeps the fastest per pass.  Until it is called the passes use the shared-memory Stockham
 * engine.  Results are identical across variants up to rounding.  The report
 * lists the timings and the choice (valid until the next ih_autotune). */
int ih_autotune(ih_context *c);
const char *ih_autotune_report(const ih_context *c);
/* Pin or read the engine of one pass: pass 0 = x, 1 = y, 2 = the fused
 * inverse x pass, 3 / 4 = the x / y derivative round trips (two-step forms
 * only), 5 = the last x pass of the tensor sources (0 = x passes then
 * update_h, 1 = one kernel accumulating the TT projection), 6 = the z passes
 * of the RHS at nz = 256 (1 = the wide-row engine, 8 lanes x 16 values per
 * row, both precisions -- the default; 2 = the same, each row's next input
 * spectrum copied into shared memory with cp.async during the current
 * transform, mixed form only; 0 = a warp per row), 7 =
 * the kz slab width of the forward y and x passes of the six tensor sources
 * (0 = whole arrays, the default; a multiple of 8 up to 64 = y then x pass on
 * one slab of all six at a time, so the slab stays in L2 between the two; it
 * applies with pass 5 = 0), 8 = the tensor sources plane-major (1: the fused
 * z pass writes each source as 129 contiguous 256 x 256 kz planes into a
 * buffer of their own, one cluster of 8 CTAs transforms a plane along y and x
 * in one pass through distributed shared memory, and update_h reads the
 * planes; 2: the same with persistent clusters that load the next plane
 * while they transform the current one; 3: persistent clusters that take
 * whole kz planes, transform the six sources of a plane one after the other
 * and accumulate their TT projection, so that update_h reads two projected
 * spectra instead of six; mixed form at 256^3 only, IH_ERR_ARG elsewhere;
 * 0: the row and column passes);
 * engine IH_FFT_STOCKHAM, IH_FFT_TWOSTEP (register two-step,
 * 128-byte tiles), IH_FFT_TWOSTEP_HALF (64-byte tiles), IH_FFT_PIPELINED
 * (register two-step in persistent CTAs that copy the next tile in with
 * cp.async while transforming the current one), IH_FFT_THREESTEP (three
 * register steps of at most 8 values; passes 0 and 1 only) or
 * IH_FFT_TWOSTEP_HALF_OCC (IH_FFT_TWOSTEP_HALF compiled for 7 resident CTAs
 * per SM; passes 0 and 1, FP32; FP64 runs IH_FFT_TWOSTEP_HALF). */
enum { IH_FFT_STOCKHAM = 0, IH_FFT_TWOSTEP = 1, IH_FFT_TWOSTEP_HALF = 2, IH_FFT_PIPELINED = 3,
       IH_FFT_THREESTEP = 4, IH_FFT_TWOSTEP_HALF_OCC = 5 };
int ih_fft_set_engine(ih_context *c, int pass, int engine);
int ih_fft_get_engine(const ih_context *c, int pass);
/* How an RHS without the filter and output flags forms the derivatives of
 * phi (on by default): 1 = round trips along x and y on the z spectrum of
 * phi (the y and x transforms that cancel are not done), 0 = from the full
 * 3-D spectrum as the filtered / output RHS does.  The two agree to
 * rounding. */
int ih_rhs_roundtrip(ih_context *c, int on);
/* DOPRI853 stage fusion (no reference counterpart; off by default): the RHS
 * evaluation of stage s also forms the input of stage s+1 (y + dt sum_j
 * a_(s+1)j k_j, dopri853.c:340-436) while it writes k_s, instead of a
 * separate combination pass that reads k_s back.  Same arithmetic in the same
 * order: results are identical to the bit either way.  It applies with the
 * separate form of the last tensor x pass (ih_fft_set_engine pass 5 = 0, the
 * autotuner's usual choice).  It saves a read of k_s per stage but the
 * update kernels that take on the combination stream up to 40 arrays at once
 * and run below the separate pass's bandwidth: at 256^3 it is slower. */
int ih_stage_fusion(ih_context *c, int on);
/* Velocity form of the DOPRI853 combinations in the mixed form (no
 * reference counterpart; on by default, no effect in FP64).  The position
 * half of every stage vector equals the velocity half of its stage input
 * (phi' = dphi, psi' = dpsi, h' = dh; toolbox.c:282-299, 311-346), so the
 * stage inputs, field_new and both error sums (dopri853.c:340-486) are formed
 * from the velocity halves alone: Y^p = y^p + dt c y^v + dt^2 (A^2 k^v),
 * field_new^p and the errors likewise with b^T A, e^T A (tableau products in
 * FP64).  Equal to the reference's combinations in exact arithmetic; the
 * position errors carry no rounding of the stage inputs.  Off: the
 * reference's formulation, as the FP64 form always uses. */
int ih_velocity_form(ih_context *c, int on);

/* CUDA graphs (no reference counterpart): each DOPRI853 try (its 11 stage
 * combinations and RHS evaluations, the final combination and the error
 * reduction) and each filtered post-step RHS without diagnostics is captured
 * once per combination of the vectors it touches and replayed as one graph
 * launch; the step size is read from device memory.  On by default; off
 * while per-kernel timing (ih_profile_enable) or the error breakdown is on.
 * Results are identical either way. */
int ih_graphs_enable(ih_context *c, int on);

/* ---- transforms (fft / ifft, toolbox.c:806-827) on host buffers ----
 * r2c unnormalised exp(-i..) [x][y][z/2+1]; c2r unnormalised exp(+i..).
 * Computed in the context's precision. */
int ih_fft_host(ih_context *c, const double *in, double *out_c);
int ih_ifft_host(ih_context *c, const double *in_c, double *out);

/* ---- initial conditions ---- */
/* Seeded fluctuations generated on the GPU: delta phi_k complex Gaussian with
 * E|c_k|^2 = amp^2/(2 omega_k L^3), omega_k = sqrt(k^2 + m^2), zero for k = 0
 * and |k| > kcut, Hermitian on the kz = 0 and kz = nz/2 planes; delta dphi_k =
 * -i omega_k delta phi_k; phi = phi0 + delta phi, dphi = dphi0 + delta dphi,
 * psi = dpsi = h = 0, a = a0.  The counter-based generator (SplitMix64 +
 * Box-Muller) makes every mode a pure function of (seed, mode index). */
int ih_ic_fluctuations(ih_context *c, uint64_t seed, double phi0,
                       double dphi0, double a0, double amp, double kcut);
/* mk_initial_psi (setup.c:825-903) on the device state. */
int ih_initial_psi(ih_context *c);

/* ---- DOPRI853 (dopri853.c) ---- */
/* initialize_dopri853 + the first RHS with filter=1 (dopri853.c:172-198,
 * toolbox.c:96-104). */
int ih_dopri853_init(ih_context *c, const ih_dopri_cfg *cfg, double t0,
                     double dt0);
/* The same with the output flag of that first RHS selectable: run_dopri853
 * opens with prepare_and_save_timeslice (dopri853.c:115, toolbox.c:96-104),
 * whose filtered RHS also computes the diagnostics (want_output = 1). */
int ih_dopri853_init_ex(ih_context *c, const ih_dopri_cfg *cfg, double t0,
                        double dt0, int want_output);
/* perform_step with dt_try; want_output=1 computes the diagnostics on the
 * post-step RHS (dopri853.c:288-291). */
int ih_dopri853_step(ih_context *c, double dt_try, int want_output,
                     ih_step_info *info);
/* The run loop (dopri853.c:112-158) to tf or max_steps accepted steps; if
 * log is not NULL, 4 doubles (t, dt_did, err, tries) per accepted step are
 * written up to log_cap steps.  *n_steps receives the accepted steps.  The
 * run ends with IH_ERR_UNDERFLOW where the reference reports a step-size
 * underflow: a try shrinking below |t| * DBL_EPSILON (perform_step,
 * dopri853.c:280-283) or a proposed step at or below dt_min
 * (MINIMAL_DELTA_T, dopri853.c:150-153; the accepted steps before it stand). */
int ih_dopri853_run(ih_context *c, double tf, long max_steps, double *log,
                    long log_cap, long *n_steps);
/* Controller state: dt_next and the number of accepted/rejected steps. */
int ih_dopri853_counters(const ih_context *c, double *dt_next, long *n_ok,
                         long *n_bad, long *n_tries);
/* Tableau (Hairer's DOP853 coefficients): c[12], a[12*12] row-major,
 * b[12], bhh[3] (stages 1, 9, 12), er[12]. */
int ih_dopri853_tableau(double *c, double *a, double *b, double *bhh,
                        double *er);
/* Dense-output coefficients of the same method (dopri853_constants.c:23-25,
 * 98-173, declared but never used by the reference's stepper):
 * ad[3*16] = the inputs of stages 14..16 over stages 1..16 (stage 13 =
 * f(field_new)), d[4*16] = the weights d4..d7 over stages 1..16. */
int ih_dopri853_dense_tableau(double *ad, double *d);
/* Dense output (no reference counterpart; the reference lands output times
 * by shortening steps, as IH_OUTPUT_INTERVAL does in the drop-in): the
 * DOP853 continuous extension (order 7) of the last accepted
 * ih_dopri853_step at t_out in [t - dt_did, t].  The first call after a step
 * evaluates stages 14..16 (three RHS evaluations); further calls within the
 * same step reuse them.  The interpolant runs from the step's start state to
 * field_new as the post-step RHS left it (filtered in place when the filter
 * is on, so with the filter it reproduces the filtered end state at t).  With
 * want_output = 1 the interpolated state then passes through the output RHS
 * of a saved slice (filtered, diagnostics kept for ih_get_output, summaries
 * of the interpolated state).  field_out (Ntot doubles, reference layout; may
 * be NULL) receives the interpolated state, after that RHS when want_output.
 * The context's own state, time and controller are unchanged.
 * IH_ERR_STATE without an accepted step since the last state change (a new
 * try, RK4 step, state upload or standalone RHS ends it); IH_ERR_ARG for
 * t_out outside the step.  Mixed form: stages 6..12 of a velocity-form step
 * get their position halves restored from the velocity halves first. */
int ih_dopri853_dense(ih_context *c, double t_out, int want_output, double *field_out);

/* ---- learned step-size proposer (no reference counterpart) ----
 * A 12 -> 64 -> 64 -> 1 MLP (GELU), BF16 weights, FP32 accumulation, trained
 * on the GPU by Adam.  Input features of accepted step n (ih_step_features):
 * log dt_n..dt_{n-3}, log err_n..err_{n-3} (accepted tries), log a, H,
 * log rms(delta phi), log rms(delta psi); output log dt_{n+1}.  With a
 * proposer set, the step size after an accepted step is its proposal (clamped
 * to [minscale, maxscale] x dt and to the Hubble cap); DOPRI853's error
 * estimate still accepts or rejects every try, and a rejected proposal is
 * reduced by the reference controller (dopri853.c:534-538). */
#define IH_MLP_INPUTS 12
#define IH_MLP_NPARAMS 5057
typedef struct ih_mlp ih_mlp;
int ih_mlp_create(int device, unsigned seed, ih_mlp **out);
void ih_mlp_destroy(ih_mlp *m);
const char *ih_mlp_last_error(const ih_mlp *m);
/* FP32 master parameters: W1[12][64], b1[64], W2[64][64], b2[64], W3[64], b3 */
int ih_mlp_set_params(ih_mlp *m, const float *params);
int ih_mlp_get_params(ih_mlp *m, float *params);
/* the BF16-rounded copy the forward and backward passes use */
int ih_mlp_get_bf16_params(ih_mlp *m, float *params);
/* x_norm = (x - in_mean) / in_std; log dt = out * out_std + out_mean */
int ih_mlp_set_norm(ih_mlp *m, const float *in_mean, const float *in_std, float out_mean,
                    float out_std);
int ih_mlp_forward(ih_mlp *m, const float *x, int n, float *y);
/* full-batch gradient of the mean squared error (normalised output units) */
int ih_mlp_gradients(ih_mlp *m, const float *x, const float *y, int n, float *grad,
                     float *loss);
/* Adam (beta 0.9 / 0.999), `iters` minibatches of `batch` <= 128 rows drawn
 * with a counter-based generator; loss_hist (iters floats) may be NULL */
int ih_mlp_train(ih_mlp *m, const float *x, const float *y, int n, int iters, int batch,
                 float lr, unsigned seed, float *loss_hist);
/* the feature vector of the last accepted step (12 floats) */
int ih_step_features(ih_context *c, float *out12);
/* set (or with NULL clear) the proposer of a context */
int ih_dopri853_set_proposer(ih_context *c, ih_mlp *m);

/* ---- ensembles (no reference counterpart: the reference runs one
 * realization per process) ----
 * An ensemble owns `count` member contexts (each its own grid, box and
 * precision; sizes as for ih_create) on one device.  Initial data
 * and outputs go through the member contexts (ih_ensemble_member).
 * ih_ensemble_run advances every member to tf with its own DOPRI853 step
 * sizes and controller (each member follows exactly the step sequence that
 * ih_dopri853_run would give it alone): in each round every unfinished
 * member queues one try -- one CUDA-graph launch on the member's own stream
 * -- before any is waited for, so the members' tries run concurrently;
 * accepted members queue their filtered post-step RHS.  *rounds and *steps
 * receive the rounds taken and the accepted steps of all members. */
typedef struct ih_ensemble ih_ensemble;
int ih_ensemble_create(const ih_params *members, int count, ih_ensemble **out);
void ih_ensemble_destroy(ih_ensemble *e);
const char *ih_ensemble_last_error(const ih_ensemble *e);
int ih_ensemble_size(const ih_ensemble *e);
ih_context *ih_ensemble_member(ih_ensemble *e, int i);
/* ih_autotune once per distinct grid and precision, shared by the members */
int ih_ensemble_autotune(ih_ensemble *e);
int ih_ensemble_dopri_init(ih_ensemble *e, const ih_dopri_cfg *cfg, double t0,
                           double dt0);
int ih_ensemble_run(ih_ensemble *e, double tf, long max_rounds, long *rounds,
                    long *steps);

/* ---- RK4 (rk4.c:27-132) ---- */
/* One step of size dt from the context time; the stage-1 RHS runs with
 * filter=1 and, if want_output, output=1 (rk4.c:63-75). */
int ih_rk4_step(ih_context *c, double dt, int want_output);
/* The state at the start of the last RK4 or DOPRI853 step as that step used
 * it (after its filter): what rk4.c's save() reads from field at an output
 * step (rk4.c:66-72), in the reference layout (Ntot doubles).  No reference
 * counterpart (the reference's field array is that state at that moment). */
int ih_get_step_start_state(ih_context *c, double *f_host);

/* Mixed form only: before an element of the two embedded error vectors enters
 * the FP64 error norm, its FP32 rounding floor eta * 2^-24 * sum_j |c_j k_j|
 * is subtracted from its magnitude (soft threshold), so that FP32 round-off
 * in the stage vectors does not drive the step size down; elements of the
 * dh segment also drop eta * 2^-24 * sum_j |c_j| max|dh'_j| (the absolute
 * noise the FP32 transforms of the tensor sources leave on every mode).
 * Default eta = 256 in the mixed form; the plain FP64 form ignores it.  No
 * reference counterpart (the reference is FP64 only). */
int ih_dopri853_set_noise_floor(ih_context *c, double eta);
/* Diagnostic: with diag on, every try also sums the squared scaled error
 * components per state segment; ih_dopri853_error_breakdown returns the last
 * try's sums [phi, dphi, psi, dpsi, h1+h2, dh1+dh2] x (S_bhh, S_er): S_bhh
 * sums (yerr/sk)^2 with yerr from the b - bhh weights (the 3rd-order
 * estimate, dopri853.c:451-452), S_er sums (yerr2/sk)^2 with the er weights
 * (the 5th-order estimate, 453-456); error() = dt * S_er / sqrt(Ntot * (S_er
 * + 0.01 S_bhh)) over all segments (dopri853.c:469-486; the scale factor's
 * share is the remainder of the totals). */
int ih_dopri853_diag_enable(ih_context *c, int on);
int ih_dopri853_error_breakdown(ih_context *c, double *out12);

/* ---- timing and instrumentation ---- */
/* Synchronise the context's stream. */
int ih_sync(ih_context *c);
/* Device time (ms, CUDA events on the context stream) accumulated by the
 * kernels of class `cls` since the last reset, and their launch count:
 * cls 0 = all FFT passes, 1 = pointwise RHS kernels, 2 = stepper kernels. */
int ih_profile_enable(ih_context *c, int on);
int ih_profile_read(ih_context *c, int cls, double *ms, long *launches);
/* The same per kernel kind (0 .. ih_profile_kernel_count()-1, named by
 * ih_profile_kernel_name), with the algorithmic bytes of the timed launches
 * (each input read once, each output written once). */
int ih_profile_kernel(ih_context *c, int kind, double *ms, long *launches,
                      double *bytes);
const char *ih_profile_kernel_name(int kind);
int ih_profile_kernel_count(void);
/* CUDA-event timer on the context stream: start, then stop returns ms. */
int ih_timer_start(ih_context *c);
int ih_timer_stop(ih_context *c, double *ms);
/* Kernel launches issued by this context since creation. */
unsigned long long ih_kernel_launches(const ih_context *c);

/* ---- pinned host memory for end-to-end transfers ---- */
int ih_host_alloc(size_t bytes, void **out);
int ih_host_free(void *p);

/* ---- measurement (no reference counterpart) ----
 * FP64 FMA throughput of GPU `device` in TFLOP/s: independent DFMA chains in
 * 8 CTAs of 256 threads per SM, `iters` links per chain, best of `reps`
 * CUDA-event-timed launches after one warm-up.  The ALU roofline of the
 * plain FP64 form. */
int ih_fp64_fma_peak(int device, int iters, int reps, double *tflops);
/* The tensor sources' plane transforms (ih_fft_set_engine pass 8: form 1 one
 * cluster per plane, 2 persistent clusters, 3 persistent clusters with the
 * TT projection, k vectors of a box of 20) alone on a zeroed buffer of six
 * 256 x 256 x mz complex FP32 spectra (mz = 129 at 256^3: 405 MB), `reps`
 * CUDA-event-timed launches after one warm-up: milliseconds per launch. */
int ih_gw_plane_probe(int device, int form, int mz, int reps, double *ms_per_launch);

#ifdef __cplusplus
}
#endif
#endif
