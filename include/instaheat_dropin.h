/*
 * instaheat_dropin.h -- the reference's own C entry points for the RHS and
 * the time steppers, implemented by the C99 layer ih_dropin.c on top of
 * libinstaheat_gpu.so (instaheat_gpu.h).
 *
 * A reference build links ih_dropin.o and libinstaheat_gpu.so in place of
 * toolbox.o, dopri853.o, dopri853_constants.o and rk4.o; main.c, setup.c and
 * io.c relink unchanged.  ih_dropin.c is compiled against the build's own
 * main.h and io.h (the reference's generated headers, or the standalone pair
 * under instaheat_gb300/dropin/host/), so it reads the same globals (pars,
 * field, dfield, rho, pressure, rho_mean, pressure_mean, tmp, mon and the
 * output structs) and the same compile-time parameters (GRIDPOINTS_*,
 * SPATIAL_*_BOUND_*, MASS, ENABLE_GW, ENABLE_FFT_FILTER, POWER_SPECTRUM_BINS,
 * the DOPRI853 controller keys, OUTPUT_*).
 *
 * Two optional keys select the GPU form: IH_PRECISION (IH_PREC_F64, the
 * default, or IH_PREC_MIXED) and IH_DEVICE (CUDA ordinal, default 0).  A
 * third, IH_OUTPUT_INTERVAL (> 0), makes run_dopri853 land steps on
 * ti + k * IH_OUTPUT_INTERVAL and write the time slices there (as its
 * overshoot clamp lands the last step on tf) instead of every
 * TIME_STEP_SKIPS steps; with a fourth, IH_DENSE_OUTPUT (1), the steps keep
 * the controller's size and each slice at ti + k * IH_OUTPUT_INTERVAL < tf
 * comes from the DOP853 continuous extension of the accepted step that
 * contains it (ih_dopri853_dense: three extra RHS evaluations per step with
 * slices, then the output RHS of the interpolated state).
 *
 * Differences from the reference functions, all on the side of what callers
 * observe after a call:
 *   - errors print a message to stderr and exit(EXIT_FAILURE), as the
 *     reference does, except step-size underflow (a message, then the run
 *     loop ends, dopri853.c:280-283);
 *   - after mk_rhs the host arrays rho, pressure and tmp.lap and the
 *     scalars rho_mean, pressure_mean hold what the reference leaves there
 *     (toolbox.c:114-127, 216-224); tmp.grad and tmp.xphi/yphi/zphi are not
 *     written (the fused GPU pass never stores the gradient components or
 *     their squared sum);
 *   - run_dopri853 / run_rk4 keep the state on the GPU and copy it to the
 *     host field / dfield arrays only when save() or the wrap-up reads them.
 */
#ifndef INSTAHEAT_DROPIN_H
#define INSTAHEAT_DROPIN_H

#include <complex.h>
#include <stddef.h>
#include <stdint.h>

#include "instaheat_gpu.h"

/* toolbox.h:15-35 (same include guard, so either header may come first) */
#ifndef __TOOLBOX__
#define __TOOLBOX__
struct evolution_flags {
    uint8_t filter; /* apply the spectral filter to the input state */
    uint8_t output; /* compute the output quantities of this time slice */
};
extern struct evolution_flags evo_flags;

void mk_rhs(const double t, double *f, double *result);
void prepare_and_save_timeslice();
void mk_gradient_squared_and_laplacian(double *in);
void mk_rho_and_p(const double *f);
void fft(double *in, complex *out);
void ifft(complex *in, double *out);
double mean(const double *f, const size_t N);
double variance(const double mean, const double *f, const size_t N);
#endif

/* dopri853.h:51, rk4.h:14 */
void run_dopri853();
void run_rk4();

/* The context behind the drop-in symbols (created on first use from pars and
 * the compile-time parameters) and its release.  No reference counterpart. */
ih_context *ih_dropin_context(void);
void ih_dropin_release(void);

#endif
