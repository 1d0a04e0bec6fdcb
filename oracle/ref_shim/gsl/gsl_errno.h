/*
 * gsl/gsl_errno.h (shim) -- GSL's status codes, as far as the reference's
 * src/setup.c tests them (setup.c:1010, 1097, 1109).  TEST INFRASTRUCTURE
 * ONLY (the second oracle, oracle/_ref); GSL is not installed here.
 */
#ifndef IH_REF_SHIM_GSL_ERRNO_H
#define IH_REF_SHIM_GSL_ERRNO_H
enum { GSL_SUCCESS = 0, GSL_FAILURE = -1, GSL_EUNIMPL = 24 };
#endif
