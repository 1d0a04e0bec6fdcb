/* Test stub: the few FFTW type names a main.h generated from InstaHeat's
 * main_template.h mentions, for a syntax-only compile of the drop-in layer
 * against that header (FFTW itself is not installed here). */
#ifndef IH_TEST_FFTW3_STUB_H
#define IH_TEST_FFTW3_STUB_H
typedef double fftw_complex[2];
typedef struct ih_test_fftw_plan_s *fftw_plan;
#endif
