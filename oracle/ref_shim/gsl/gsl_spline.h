/*
 * gsl/gsl_spline.h (shim) -- declarations of the GSL cubic-spline calls in
 * the reference's Bunch-Davies initial conditions (setup.c:1007-1035).  TEST
 * INFRASTRUCTURE ONLY (the second oracle, oracle/_ref); never reached with
 * IC_FROM_DAT_FILE_* data, and defined to report that they are absent.
 */
#ifndef IH_REF_SHIM_GSL_SPLINE_H
#define IH_REF_SHIM_GSL_SPLINE_H

#include <stddef.h>
#include "gsl_errno.h"

typedef struct { const char *name; } gsl_interp_type;
typedef struct gsl_interp_accel gsl_interp_accel;
typedef struct gsl_spline gsl_spline;

extern const gsl_interp_type *gsl_interp_cspline;

gsl_interp_accel *gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel *a);
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t size);
int gsl_spline_init(gsl_spline *spline, const double xa[], const double ya[], size_t size);
double gsl_spline_eval(const gsl_spline *spline, double x, gsl_interp_accel *a);
void gsl_spline_free(gsl_spline *spline);

#endif
