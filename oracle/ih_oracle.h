/*
 * ih_oracle.h -- CPU oracle for the InstaHeat RHS + DOPRI853/RK4 hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C99 + OpenMP restatement of the
 * reference algorithm (nikikilbertus/InstaHeat, src/toolbox.c, src/dopri853.c,
 * src/rk4.c and the k-grid / filter / psi-constraint parts of src/setup.c).
 * It exists to check the CUDA library and to time a CPU baseline.  Only the
 * test-suite, the smoke check and the benchmark's CPU-baseline leg may load it;
 * the product library never links, calls or falls back to it.
 *
 * Parity pin: the reference ships no golden vectors.  The oracle is pinned
 * against the known answers the reference's own validation material defines
 * (evaluation/testLaplacian.m: spectral derivatives of sin x sin y sin z;
 * helpers/flrw_homogeneous.py: the homogeneous FLRW background, imported from
 * the reference to make tests/golden/flrw_*.json; evaluation/mkPowerSpectrum.m:
 * the shell-binning rule; the DOPRI853 order conditions), and against an
 * independent numpy restatement (oracle/rhs_numpy.py, pocketfft).
 *
 * Layout conventions follow the reference (src/main_template.h:223-233):
 * state f[Ntot], Ntot = 4N + 4Next + 1, order phi, dphi, psi, dpsi (N reals,
 * row-major [x][y][z]), h1, h2, dh1, dh2 (Next = 2M doubles = M interleaved
 * complex, r2c half spectrum [x][y][z/2+1]), then the scale factor a.
 */
#ifndef IH_ORACLE_H
#define IH_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny, nz;          /* grid points, nx >= ny >= nz, 3D, nz even */
    double lx, ly, lz;       /* box lengths (SPATIAL_UPPER - SPATIAL_LOWER) */
    double mass;             /* MASS: V = m^2 phi^2 / 2 */
    int gw;                  /* ENABLE_GW */
    int filter;              /* ENABLE_FFT_FILTER */
    int bins;                /* POWER_SPECTRUM_BINS (also the GW spectrum) */
    int threads;             /* OpenMP threads, <= 0: all */
} iho_params;

/* Diagnostics computed when the output flag is set (toolbox.c:251-270). */
typedef struct {
    double *phi_ps, *psi_ps, *rho_ps, *gw; /* bins each */
    double cstr[4];          /* ham l2 (mean of squares), ham max, mom l2, mom max */
    double smry[6][4];       /* phi, dphi, psi, dpsi, rho, p: mean, var, min, max */
} iho_output;

typedef struct iho_ctx iho_ctx;

/* Sizes (setup.c:228-271). */
void iho_sizes(int nx, int ny, int nz, size_t *N, size_t *M, size_t *Next,
               size_t *Ntot);

iho_ctx *iho_create(const iho_params *p);
void iho_destroy(iho_ctx *c);

/* k grids (setup.c:609-666): 7 arrays of M doubles, k_max. */
void iho_kgrid(const iho_ctx *c, double *kx, double *ky, double *kz,
               double *kxf, double *kyf, double *kzf, double *ksq,
               double *kmax);
/* Filter mask (setup.c:710-754). */
void iho_filter_mask(const iho_ctx *c, double *mask);

/* 3D FFTs with FFTW's conventions: r2c unnormalised exp(-i..), c2r
 * unnormalised exp(+i..).  Complex arrays are interleaved re/im. */
void iho_fft(iho_ctx *c, const double *in, double *out_c);
void iho_ifft(iho_ctx *c, const double *in_c, double *out);

/* mk_rhs (toolbox.c:75-88).  filter/output are evo_flags; with filter=1 the
 * input state is overwritten by its filtered version (toolbox.c:164-171).
 * out may be NULL when output=0. */
void iho_mk_rhs(iho_ctx *c, double t, double *f, double *result,
                int filter, int output, iho_output *out);
double iho_rho_mean(const iho_ctx *c);
double iho_pressure_mean(const iho_ctx *c);
const double *iho_rho(const iho_ctx *c);
const double *iho_pressure(const iho_ctx *c);
const double *iho_lap(const iho_ctx *c);
const double *iho_grad2(const iho_ctx *c);
unsigned long iho_calls_rhs(const iho_ctx *c);

/* mk_initial_psi (setup.c:825-903): overwrite psi, dpsi of f from phi, dphi, a. */
void iho_initial_psi(iho_ctx *c, double *f, double t);

double iho_mean(const double *f, size_t n);
double iho_variance(double mean, const double *f, size_t n);

/* ---- DOPRI853 (dopri853.c) ---- */
typedef struct {
    double rtol, atol;       /* RELATIVE_TOLERANCE, ABSOLUTE_TOLERANCE */
    double beta, safe;       /* BETA, SAFE */
    double minscale, maxscale; /* SMALLEST_SCALING, LARGEST_SCALING */
    double max_dt_hubble_fraction; /* <= 0: no cap */
    double dt_min;           /* MINIMAL_DELTA_T */
    double max_steps;        /* MAX_STEPS */
} iho_dopri_cfg;

typedef struct {
    double t, dt, dt_next, dt_did, err_old;
    int reject;
    long n_stp, n_ok, n_bad;
    double last_err;         /* error() of the last try */
    long tries;              /* total try_step calls */
} iho_dopri_state;

/* Tableau accessor for order-condition tests: c[12], a[12][12], b[12],
 * bhh[3] (stages 1, 9, 12), er[12]. */
void iho_dopri853_tableau(double *c, double *a, double *b, double *bhh,
                          double *er);

/* Initialise: state->t = t0, dt = dt0; computes dfield = rhs(field) with
 * filter=1 and output=0 like prepare_and_save_timeslice (toolbox.c:96-104). */
/* the dense-output coefficients (dopri853_constants.c:23-25, 98-173):
   ad[3][16] = inputs of stages 14..16 over stages 1..16 (stage 13 =
   f(field_new)), d[4][16] = d4..d7 over stages 1..16 */
void iho_dopri853_dense_tableau(double *ad, double *d);
void iho_dopri853_init(iho_ctx *c, const iho_dopri_cfg *cfg,
                       iho_dopri_state *st, double *field, double *dfield,
                       double t0, double dt0);
/* perform_step (dopri853.c:271-311); returns 0 ok, 1 underflow.  field and
 * dfield are advanced in place.  out != NULL requests output on the post-step
 * RHS. */
int iho_dopri853_step(iho_ctx *c, const iho_dopri_cfg *cfg,
                      iho_dopri_state *st, double *field, double *dfield,
                      double dt_try, iho_output *out);
/* iho_dopri853_step (no output flag), then the DOP853 continuous extension
   of the accepted step at the n fractions theta[q] of it (0 = the step's
   start, 1 = its end): dense_out[q * Ntot + i].  Three extra RHS
   evaluations (stages 14-16). */
int iho_dopri853_step_dense(iho_ctx *c, const iho_dopri_cfg *cfg,
                            iho_dopri_state *st, double *field, double *dfield,
                            double dt_try, int n, const double *theta,
                            double *dense_out);
/* run loop (dopri853.c:112-158) from st->t to tf, capped at max_steps; the
 * step log (t, dt_did, err, accepted) is written to log[4*k] when log is not
 * NULL and k < log_cap.  Returns number of accepted steps. */
long iho_dopri853_run(iho_ctx *c, const iho_dopri_cfg *cfg,
                      iho_dopri_state *st, double *field, double *dfield,
                      double tf, long max_steps, double *log, long log_cap);

/* ---- RK4 (rk4.c:27-132) ---- */
/* One RK4 step of size dt from t: stage-1 RHS with filter=1 (rk4.c:63-75). */
void iho_rk4_step(iho_ctx *c, double *field, double t, double dt);

/* ---- Initial conditions ---- */
/* Seeded Bunch-Davies-like fluctuations: delta phi_k complex Gaussian with
 * E|c_k|^2 = amp^2 / (2 omega_k L^3), omega_k = sqrt(k^2 + m^2), zero for
 * |k| > kcut; delta dphi_k = -i omega_k delta phi_k.  phi = phi0 + delta phi,
 * dphi = dphi0 + delta dphi, psi = dpsi = 0, h = 0, a = a0.  The Gaussian
 * deviates come from the SplitMix64-driven generator ih_normal_pair(), which
 * the CUDA library shares, so both sides consume identical states. */
void iho_ic_fluctuations(iho_ctx *c, double *f, unsigned long long seed,
                         double phi0, double dphi0, double a0, double amp,
                         double kcut);

#ifdef __cplusplus
}
#endif
#endif
