/*
 * ref_harness.c -- entry points into nikikilbertus/InstaHeat's own code for
 * the second oracle (oracle/_ref).  TEST INFRASTRUCTURE ONLY.
 *
 * oracle/ref.py compiles the reference's src/toolbox.c, setup.c, io.c,
 * rk4.c, dopri853_constants.c and main.c unmodified (main renamed to
 * ihref_main so the library can also run the whole program), against the
 * shims in oracle/ref_shim/ and a main.h rendered from src/main_template.h,
 * together with this file.  This file #includes src/dopri853.c itself, so the
 * run loop's static steps (initialize_dopri853, write_start_info,
 * perform_step, free_dopri853; dopri853.c:112-311) can be driven one step at
 * a time from Python.  Nothing here changes what those functions compute.
 */
#include "main.h"
#include "toolbox.h"
#include "setup.h"
#include "io.h"

#if INTEGRATION_METHOD == DOPRI853
#include "dopri853.c"
#elif INTEGRATION_METHOD == RK4
#include "rk4.h"
#endif

/* allocate_and_init_all (setup.c:89-108): parameters, arrays, plans, k grid,
 * filter mask, initial conditions (including the psi solve for
 * IC_FROM_DAT_FILE_WITHOUT_PSI), output file. */
void ihref_init(void) { allocate_and_init_all(); }

/* free_and_destroy_all (setup.c:1511-1516): writes the output file. */
void ihref_free(void) { free_and_destroy_all(); }

/* N, M, Next, Ntot, dim, POWER_SPECTRUM_BINS */
void ihref_sizes(size_t *out)
{
    out[0] = pars.N;
    out[1] = pars.M;
    out[2] = pars.Next;
    out[3] = pars.Ntot;
    out[4] = pars.dim;
    out[5] = POWER_SPECTRUM_BINS;
}

/* The time parameters the steppers read (pars.t, main_template.h:188-195). */
void ihref_set_time(double ti, double tf, double dt)
{
    pars.t.ti = ti;
    pars.t.t = ti;
    pars.t.tf = tf;
    pars.t.dt = dt;
}

double ihref_time(void) { return pars.t.t; }

/* tmp.lap, tmp.f after mk_rhs (toolbox.c:129-186) */
double *ihref_lap(void) { return tmp.lap; }
double *ihref_tmp_f(void) { return tmp.f; }

int ihref_method(void) { return INTEGRATION_METHOD; }

#if INTEGRATION_METHOD == DOPRI853
/* run_dopri853's prologue (dopri853.c:114-116): controller set-up, work
 * vectors, tolerances, and the first prepare_and_save_timeslice, which
 * filters the state in place and fills dfield. */
void ihref_dopri_begin(void)
{
    initialize_dopri853();
    write_start_info();
    prepare_and_save_timeslice();
}

/* One perform_step (dopri853.c:271-311) from the current state; out receives
 * t, dt_did, dt_next, err_old, reject.  Returns perform_step's status (1 on
 * step-size underflow). */
int ihref_dopri_step(double dt_try, double *out)
{
    const int st = perform_step(dt_try);
    out[0] = dp.t;
    out[1] = dp.dt_did;
    out[2] = dp.dt_next;
    out[3] = dp.err_old;
    out[4] = (double)dp.reject;
    return st;
}

void ihref_dopri_end(void) { free_dopri853(); }
#endif
