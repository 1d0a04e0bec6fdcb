/*
 * gsl/gsl_integration.h (shim) -- declarations of the GSL quadrature calls in
 * the reference's Bunch-Davies kernel (setup.c:1070-1120).  TEST
 * INFRASTRUCTURE ONLY (the second oracle, oracle/_ref).  The oracle drives the
 * reference with IC_FROM_DAT_FILE_* initial data, which never reaches these
 * calls; they are defined to print a message and return GSL_EUNIMPL, so a
 * Bunch-Davies build stops at the reference's own error check.
 */
#ifndef IH_REF_SHIM_GSL_INTEGRATION_H
#define IH_REF_SHIM_GSL_INTEGRATION_H

#include <stddef.h>
#include "gsl_errno.h"

typedef struct {
    double (*function)(double x, void *params);
    void *params;
} gsl_function;

typedef struct gsl_integration_workspace gsl_integration_workspace;
typedef struct gsl_integration_qawo_table gsl_integration_qawo_table;
enum gsl_integration_qawo_enum { GSL_INTEG_COSINE, GSL_INTEG_SINE };

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
gsl_integration_qawo_table *gsl_integration_qawo_table_alloc(
    double omega, double L, enum gsl_integration_qawo_enum sine, size_t n);
int gsl_integration_qawo_table_set(gsl_integration_qawo_table *t, double omega, double L,
                                   enum gsl_integration_qawo_enum sine);
void gsl_integration_qawo_table_free(gsl_integration_qawo_table *t);
int gsl_integration_qagiu(gsl_function *f, double a, double epsabs, double epsrel,
                          size_t limit, gsl_integration_workspace *workspace,
                          double *result, double *abserr);
int gsl_integration_qawf(gsl_function *f, const double a, const double epsabs,
                         const size_t limit, gsl_integration_workspace *workspace,
                         gsl_integration_workspace *cycle_workspace,
                         gsl_integration_qawo_table *wf, double *result, double *abserr);

#endif
