/*
 * ih_dropin.c -- InstaHeat's toolbox and stepper entry points (toolbox.h:15-35,
 * dopri853.h:51, rk4.h:14) in C99 on top of libinstaheat_gpu.so.
 *
 * Compiled against the host build's main.h / io.h: the reference's generated
 * headers when it replaces toolbox.c, dopri853.c, dopri853_constants.c and
 * rk4.c in a reference build, or the standalone pair in host/.  Reads the
 * same globals and compile-time parameters as the files it replaces; see
 * include/instaheat_dropin.h for what differs.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "main.h"
#include "io.h"
#include "instaheat_dropin.h"

#ifndef IH_PRECISION
#define IH_PRECISION IH_PREC_F64
#endif
#ifndef IH_DEVICE
#define IH_DEVICE 0
#endif

struct evolution_flags evo_flags = {.filter = 0, .output = 0};

static ih_context *ctx_ = NULL;
static double *scratch_ = NULL; /* Ntot doubles: RHS results a caller discards */

static void fail(const char *where, int st)
{
    fprintf(stderr, "%s: %s%s%s\n", where, ih_status_string(st), ctx_ ? ": " : "",
            ctx_ ? ih_last_error(ctx_) : "");
    exit(EXIT_FAILURE);
}

#define IH_CHECK(where, call)                                                  \
    do {                                                                       \
        int st_ = (call);                                                      \
        if (st_ != IH_OK) fail(where, st_);                                    \
    } while (0)

ih_context *ih_dropin_context(void)
{
    if (ctx_) {
        return ctx_;
    }
    ih_params p;
    memset(&p, 0, sizeof p);
    p.nx = (int)pars.x.N;
    p.ny = (int)pars.y.N;
    p.nz = (int)pars.z.N;
    p.lx = pars.x.b - pars.x.a;
    p.ly = pars.y.b - pars.y.a;
    p.lz = pars.z.b - pars.z.a;
    p.mass = MASS;
#ifdef ENABLE_GW
    p.enable_gw = 1;
#endif
#ifdef ENABLE_FFT_FILTER
    p.enable_filter = 1;
#endif
    p.bins = POWER_SPECTRUM_BINS;
    p.precision = IH_PRECISION;
    p.device = IH_DEVICE;
    int st = ih_create(&p, &ctx_);
    if (st != IH_OK) {
        /* ih_create leaves no context behind on failure */
        ctx_ = NULL;
        fprintf(stderr, "ih_create (%zu x %zu x %zu): %s\n", pars.x.N, pars.y.N, pars.z.N,
                ih_status_string(st));
        exit(EXIT_FAILURE);
    }
    scratch_ = malloc(pars.Ntot * sizeof *scratch_);
    if (!scratch_) {
        fputs("Allocating memory failed.\n", stderr);
        exit(EXIT_FAILURE);
    }
    return ctx_;
}

void ih_dropin_release(void)
{
    if (ctx_) {
        ih_destroy(ctx_);
        ctx_ = NULL;
    }
    free(scratch_);
    scratch_ = NULL;
}

/* what mk_rhs leaves in host globals (toolbox.c:114-127, 216-224) */
static void mirror_rhs(ih_context *c)
{
    IH_CHECK("mk_rhs", ih_get_means(c, &rho_mean, &pressure_mean));
    IH_CHECK("mk_rhs", ih_get_field(c, 0, rho));
    IH_CHECK("mk_rhs", ih_get_field(c, 1, pressure));
    IH_CHECK("mk_rhs", ih_get_field(c, 2, tmp.lap));
}

/* the output buffers that output_all fills (toolbox.c:251-270) */
static void fill_outputs(ih_context *c)
{
    ih_output o;
    memset(&o, 0, sizeof o);
#ifdef OUTPUT_PHI_PS
    o.phi_ps = phi_ps.tmp;
#endif
#ifdef OUTPUT_PSI_PS
    o.psi_ps = psi_ps.tmp;
#endif
#ifdef OUTPUT_RHO_PS
    o.rho_ps = rho_ps.tmp;
#endif
#ifdef ENABLE_GW
    o.gw = gw.tmp;
#endif
    IH_CHECK("output", ih_get_output(c, &o));
#ifdef OUTPUT_CONSTRAINTS
    memcpy(cstr.tmp, o.cstr, sizeof o.cstr);
#endif
#ifdef OUTPUT_PHI_SMRY
    memcpy(phi_smry.tmp, o.smry[0], sizeof o.smry[0]);
#endif
#ifdef OUTPUT_DPHI_SMRY
    memcpy(dphi_smry.tmp, o.smry[1], sizeof o.smry[1]);
#endif
#ifdef OUTPUT_PSI_SMRY
    memcpy(psi_smry.tmp, o.smry[2], sizeof o.smry[2]);
#endif
#ifdef OUTPUT_DPSI_SMRY
    memcpy(dpsi_smry.tmp, o.smry[3], sizeof o.smry[3]);
#endif
#ifdef OUTPUT_RHO_SMRY
    memcpy(rho_smry.tmp, o.smry[4], sizeof o.smry[4]);
#endif
#ifdef OUTPUT_PRESSURE_SMRY
    memcpy(p_smry.tmp, o.smry[5], sizeof o.smry[5]);
#endif
#ifdef OUTPUT_RHO
    IH_CHECK("output", ih_get_field(c, 0, rho));
#endif
}

void mk_rhs(const double t, double *f, double *result)
{
    ih_context *c = ih_dropin_context();
    IH_CHECK("mk_rhs", ih_mk_rhs_host(c, t, f, result, evo_flags.filter, evo_flags.output));
    mon.calls_rhs += 1;
    mirror_rhs(c);
    if (evo_flags.output == 1) {
        fill_outputs(c);
    }
}

void prepare_and_save_timeslice()
{
    evo_flags.output = 1;
    evo_flags.filter = 1;
    mk_rhs(pars.t.t, field, dfield);
    evo_flags.filter = 0;
    evo_flags.output = 0;
    save();
}

/* Both run one RHS evaluation of `in` (the GPU pipeline forms the gradient,
 * the Laplacian, rho and p together) and keep its side effects; the result
 * itself is discarded. */
void mk_gradient_squared_and_laplacian(double *in)
{
    ih_context *c = ih_dropin_context();
    IH_CHECK("mk_gradient_squared_and_laplacian",
             ih_mk_rhs_host(c, pars.t.t, in, scratch_, evo_flags.filter, 0));
    IH_CHECK("mk_gradient_squared_and_laplacian", ih_get_field(c, 2, tmp.lap));
}

void mk_rho_and_p(const double *f)
{
    ih_context *c = ih_dropin_context();
    /* filter = 0: the input is read only */
    IH_CHECK("mk_rho_and_p", ih_mk_rhs_host(c, pars.t.t, (double *)f, scratch_, 0, 0));
    mirror_rhs(c);
}

void fft(double *in, complex *out)
{
    IH_CHECK("fft", ih_fft_host(ih_dropin_context(), in, (double *)out));
}

void ifft(complex *in, double *out)
{
    IH_CHECK("ifft", ih_ifft_host(ih_dropin_context(), (const double *)in, out));
}

double mean(const double *f, const size_t N)
{
    double m = 0.0;
    IH_CHECK("mean", ih_mean_host(ih_dropin_context(), f, N, &m));
    return m;
}

double variance(const double mean, const double *f, const size_t N)
{
    double v = 0.0;
    IH_CHECK("variance", ih_variance_host(ih_dropin_context(), mean, f, N, &v));
    return v;
}

static ih_dopri_cfg controller(void)
{
    ih_dopri_cfg cfg;
    cfg.rtol = RELATIVE_TOLERANCE;
    cfg.atol = ABSOLUTE_TOLERANCE;
    cfg.beta = BETA;
    cfg.safe = SAFE;
    cfg.minscale = SMALLEST_SCALING;
    cfg.maxscale = LARGEST_SCALING;
    cfg.max_dt_hubble_fraction = MAX_DT_HUBBLE_FRACTION;
    cfg.dt_min = MINIMAL_DELTA_T;
    cfg.max_steps = (double)MAX_STEPS;
    return cfg;
}

/* dopri853.c:112-158 with the state on the GPU; the host field (and dfield)
 * arrays are brought up to date whenever save() or the wrap-up reads them. */
void run_dopri853()
{
    ih_context *c = ih_dropin_context();
    const ih_dopri_cfg cfg = controller();
    const double tf = pars.t.tf;
    double t = pars.t.ti, dt = pars.t.dt;
    const unsigned long long calls0 = ih_calls_rhs(c);

    INFO(puts("Initialized dopri853 parameters.\n"));
    INFO(puts("Starting dopri853 integration with:"));
    INFO(printf("  Initial time: %.17g\n", pars.t.ti));
    INFO(printf("  Final time: %.17g\n", tf));
    INFO(printf("  Initial time step dt: %.17g\n", dt));
    INFO(printf("  Minimal time step dt: %.17g\n", (double)MINIMAL_DELTA_T));
    INFO(printf("  Max number of steps: %zu\n", (size_t)MAX_STEPS));
    INFO(printf("  Relative tolerance: %.17g\n", (double)RELATIVE_TOLERANCE));
    INFO(printf("  Absolute tolerance: %.17g\n\n", (double)ABSOLUTE_TOLERANCE));

    /* initialize_dopri853 + prepare_and_save_timeslice on the device state */
    IH_CHECK("run_dopri853", ih_set_state(c, field, t));
    pars.t.t = t;
    IH_CHECK("run_dopri853", ih_dopri853_init_ex(c, &cfg, t, dt, 1));
    IH_CHECK("run_dopri853", ih_get_state(c, field));
    IH_CHECK("run_dopri853", ih_get_dstate(c, dfield));
    fill_outputs(c);
    t_out.tmp[0] = t;
    save();

    TIME(mon.integration = -get_wall_time());
    size_t n_stp, n_ok = 0, n_bad = 0;
#ifdef IH_OUTPUT_INTERVAL
    /* output landing: steps are shortened to end on ti + k * interval, and
     * the slices are written there instead of every TIME_STEP_SKIPS steps;
     * with IH_DENSE_OUTPUT (1) the steps keep their size and the slices come
     * from the continuous extension of the step that contains them */
#if defined(IH_DENSE_OUTPUT)
    const int dense = (IH_DENSE_OUTPUT) != 0;
#else
    const int dense = 0;
#endif
    size_t n_out = 1;
    double t_out_next = pars.t.ti + (double)n_out * IH_OUTPUT_INTERVAL;
#endif
    for (n_stp = 0;; ++n_stp) {
        if (t + dt * 1.0001 > tf) {
            dt = tf - t;
            INFO(printf("\nOvershoot, new dt = %f\n", dt));
        }
#ifdef IH_OUTPUT_INTERVAL
        int out = 0;
        if (!dense && t_out_next < tf && t + dt * 1.0001 > t_out_next) {
            dt = t_out_next - t;
            out = 1;
        }
#else
        const int out = ((n_stp + 1) % pars.file.skip == 0);
#endif
        ih_step_info info;
        const int st = ih_dopri853_step(c, dt, out, &info);
        if (st == IH_ERR_UNDERFLOW) {
            fputs("\n!!! Stepsize underflow.\n", stderr);
            break;
        }
        if (st != IH_OK) {
            fail("run_dopri853", st);
        }
        if (info.dt_did == dt) {
            ++n_ok;
        } else {
            ++n_bad;
        }
        t = info.t;
        pars.t.t = t;
        t_out.tmp[0] = t;
#ifdef IH_OUTPUT_INTERVAL
        while (dense && t_out_next < tf && t_out_next <= t) {
            IH_CHECK("run_dopri853", ih_dopri853_dense(c, t_out_next, 1, field));
            fill_outputs(c);
            pars.t.t = t_out_next;
            t_out.tmp[0] = t_out_next;
            save();
            ++n_out;
            t_out_next = pars.t.ti + (double)n_out * IH_OUTPUT_INTERVAL;
            pars.t.t = t;
            t_out.tmp[0] = t;
        }
        /* a rejected landing try ends short of the output time: no slice */
        if (out && fabs(t - t_out_next) <= 1e-12 * fmax(1.0, fabs(t_out_next))) {
            IH_CHECK("run_dopri853", ih_get_state(c, field));
            fill_outputs(c);
            save();
            ++n_out;
            t_out_next = pars.t.ti + (double)n_out * IH_OUTPUT_INTERVAL;
        }
#else
        if (out) {
            IH_CHECK("run_dopri853", ih_get_state(c, field));
            fill_outputs(c);
            save();
        }
#endif
        if (t >= tf) {
            puts("\nReached specified final time.\n");
            break;
        }
        if (n_stp >= (size_t)MAX_STEPS) {
            puts("\nReached maximal number of steps.\n");
            break;
        }
        if (get_wall_time() + mon.total > pars.max_runtime) {
            puts("\nReached specified maximal runtime.\n");
            break;
        }
        if (fabs(info.dt_next) <= MINIMAL_DELTA_T) {
            puts("\n!!! Stepsize underflow.\n");
            break;
        }
        dt = info.dt_next;
    }
    TIME(mon.integration += get_wall_time());
    mon.calls_rhs += ih_calls_rhs(c) - calls0;
    IH_CHECK("run_dopri853", ih_get_state(c, field));
    IH_CHECK("run_dopri853", ih_get_dstate(c, dfield));

    /* wrap_up_dopri853 (dopri853.c:207-233) */
    const size_t index = pars.file.index;
    if (index != 0 && t_out.buf[index - 1] < t) {
        prepare_and_save_timeslice();
    }
#ifdef ENABLE_FOLLOWUP
    h5_write_followup();
#endif
    double val[1];
    val[0] = (double)n_stp;
    h5_write_simple(H5_STEPS_TOTAL_NAME, val, 1, H5D_COMPACT);
    val[0] = (double)n_ok;
    h5_write_simple(H5_STEPS_OK_NAME, val, 1, H5D_COMPACT);
    val[0] = (double)n_bad;
    h5_write_simple(H5_STEPS_BAD_NAME, val, 1, H5D_COMPACT);
    INFO(puts("Finished dopri853:"));
#ifdef ENABLE_TIMING
    INFO(printf("  Time: %f seconds\n", mon.integration));
    h5_write_simple(H5_RUNTIME_STEPPER_NAME, &mon.integration, 1, H5D_COMPACT);
#endif
    INFO(printf("  Total steps: %zu\n", n_stp + 1));
    INFO(printf("  Good steps:  %zu\n", n_ok));
    INFO(printf("  Bad steps:   %zu\n\n", n_bad));
}

/* rk4.c:27-132 with the state on the GPU.  At an output step save() reads the
 * filtered state at the step's start time, as rk4.c does between the stage-1
 * RHS and the update. */
void run_rk4()
{
    ih_context *c = ih_dropin_context();
    const size_t Nt = pars.t.Nt;
    double dt = pars.t.dt;
    double t = pars.t.t;
    const unsigned long long calls0 = ih_calls_rhs(c);

    INFO(puts("Starting RK4 time evolution with:"));
    INFO(printf("initial time: %f\n", pars.t.ti));
    INFO(printf("final time: %f\n", pars.t.tf));
    INFO(printf("time step dt: %f\n", dt));
    INFO(printf("number of steps: %zu\n", Nt));
    (void)Nt;

#ifdef ENABLE_TIMING
    /* the reference's rk4.c declares this inside TIME(), which its own
       main.h wraps in a do-while scope: that does not compile there */
    double secs = -get_wall_time();
#endif
    IH_CHECK("run_rk4", ih_set_state(c, field, t));
    for (size_t nt = 0; t < pars.t.tf && nt < (size_t)MAX_STEPS; ++nt) {
        if (t + dt * 1.0001 > pars.t.tf) {
            dt = pars.t.tf - t;
            pars.t.dt = dt;
            INFO(printf("overshoot, new dt = %f\n", dt));
        }
        const int out = (nt % pars.file.skip == 0);
        IH_CHECK("run_rk4", ih_rk4_step(c, dt, out));
        if (out) {
            IH_CHECK("run_rk4", ih_get_step_start_state(c, field));
            fill_outputs(c);
            save();
        }
        t += dt;
        pars.t.t = t;
        t_out.tmp[0] = t;
    }
    mon.calls_rhs += ih_calls_rhs(c) - calls0;
    IH_CHECK("run_rk4", ih_get_state(c, field));

    /* make sure to write out last time slice */
    prepare_and_save_timeslice();
    if (fabs(pars.t.tf - pars.t.t) > 1e-14) {
        INFO(puts("The time of the last step does not coincide "
                  "with the specified final time."));
    }
    INFO(puts("Finished rk4"));
#ifdef ENABLE_TIMING
    secs += get_wall_time();
    INFO(printf("time: %f seconds\n\n", secs));
    double val[1] = {secs};
    h5_write_simple(H5_RUNTIME_STEPPER_NAME, val, 1, H5D_COMPACT);
#endif
}
