/*
 * fftw3.h (shim) -- the subset of FFTW3's API that nikikilbertus/InstaHeat's
 * src/ C files call, backed by the oracle's FP64 transforms (ih_oracle_fft.c).
 *
 * TEST INFRASTRUCTURE ONLY.  It exists so that the reference's own sources
 * compile and run unmodified as a second oracle (oracle/_ref); the product
 * library never includes it.  FFTW3 itself is a third-party library the
 * reference links (src/Makefile:7) but does not vendor or pin.
 *
 * Calls covered (setup.c:137-151, 524-554, 560-594, 1521-1532;
 * toolbox.c:806-827): fftw_plan_dft_{r2c,c2r}_{1,2,3}d, fftw_execute,
 * fftw_execute_dft_r2c/c2r (new-array execution on equally aligned arrays),
 * fftw_destroy_plan, fftw_malloc/fftw_free, fftw_alignment_of,
 * fftw_init_threads, fftw_plan_with_nthreads, fftw_cleanup_threads.
 *
 * Conventions kept from FFTW: r2c is the unnormalised forward DFT
 * (exp(-2 pi i jk/n)) into the half spectrum [n0][n1][n2/2+1]; c2r is the
 * unnormalised inverse of the Hermitian half spectrum.  Unlike FFTW's c2r,
 * this one leaves its input intact (FFTW may overwrite it; no caller in the
 * reference reads it afterwards).  Planner flags are accepted and ignored:
 * there is one algorithm.
 */
#ifndef IH_REF_SHIM_FFTW3_H
#define IH_REF_SHIM_FFTW3_H

#include <stddef.h>

/* fftw_complex is C99 double complex when <complex.h> came first, as FFTW's
 * own header arranges (every reference file includes complex.h before it). */
#if defined(_Complex_I) && defined(complex) && defined(I)
typedef double _Complex fftw_complex;
#else
typedef double fftw_complex[2];
#endif

typedef struct ih_ref_fftw_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)

#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_CONSERVE_MEMORY (1U << 2)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_WISDOM_ONLY (1U << 21)

fftw_plan fftw_plan_dft_r2c_1d(int n0, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_c2r_1d(int n0, fftw_complex *in, double *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out,
                               unsigned flags);

void fftw_execute(const fftw_plan p);
void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out);
void fftw_destroy_plan(fftw_plan p);

void *fftw_malloc(size_t n);
void fftw_free(void *p);
int fftw_alignment_of(double *p);

int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);

#endif
