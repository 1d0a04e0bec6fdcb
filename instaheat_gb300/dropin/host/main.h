/*
 * main.h (standalone host) -- the compile-time parameters, global structures
 * and globals that the drop-in layer (ih_dropin.c) and this host program
 * share, for builds without the reference's generated main.h.
 *
 * The member names are those of the reference's structs (main_template.h:
 * 172-287, the globals 313-355) so that ih_dropin.c compiles unchanged
 * against either header; only the members these two programs use are
 * declared, and there is no FFTW or HDF5 dependency.  The parameter values
 * come from ih_parameters.h, generated from a parameters.sh file by
 * instaheat_gb300/dropin/params.py.
 */
#ifndef __MAIN__
#define __MAIN__

#include <complex.h>
#include <stddef.h>
#include <stdint.h>

#define PI                      (3.141592653589793238462643383279)
#define TWOPI                   (6.283185307179586476925286766559)
#define MAX(x, y)               (((x) > (y)) ? (x) : (y))
#define MIN(x, y)               (((x) > (y)) ? (y) : (x))

#define SHOW_RUNTIME_INFO
#ifdef SHOW_RUNTIME_INFO
#define INFO(f) do { (f); } while (0)
#else
#define INFO(f)
#endif

/* integration methods and initial-condition kinds (the values are the
 * reference's, so parameter files mean the same thing) */
#define RK4                 (0)
#define RKF45               (1)
#define RKCK                (2)
#define DOPRI89             (3)
#define DOPRI853            (4)
#define IC_FROM_INTERNAL_FUNCTION       (0)
#define IC_FROM_H5_FILE                 (1)
#define IC_FROM_DAT_FILE_WITH_PSI       (2)
#define IC_FROM_DAT_FILE_WITHOUT_PSI    (3)
#define IC_FROM_BUNCH_DAVIES            (4)

#include "ih_parameters.h"

#ifdef ENABLE_TIMING
#define TIME(f) do { (f); } while (0)
#else
#define TIME(f)
#endif

#ifndef ENABLE_GW
#undef OUTPUT_H1_SMRY
#undef OUTPUT_H2_SMRY
#endif
#if defined(OUTPUT_PHI) || defined(OUTPUT_DPHI) || defined(OUTPUT_PSI) || \
    defined(OUTPUT_DPSI) || defined(OUTPUT_RHO)
#define LARGE_OUTPUT
#endif

struct grid_dimension {
    size_t N;       /* grid points in real space */
    size_t M;       /* grid points in Fourier space */
    double a, b;    /* interval [a, b) */
    double k, k2;   /* 2 pi / (b - a) and its square */
    size_t stride;  /* output stride */
    size_t outN;    /* output points */
};

struct timing {
    size_t Nt;      /* steps of a fixed-step run */
    double dt, ti, tf, t;
};

struct output {
    size_t dim;     /* values per time slice */
    size_t id;      /* dataset index in the output container */
    double *buf;    /* WRITE_OUT_BUFFER_NUMBER slices */
    double *tmp;    /* the current slice */
};

struct file_parameters {
    size_t id, index, buf_size, skip;
};

struct parameters {
    struct grid_dimension x, y, z;
    size_t N, Next, Ntot, outN, M, dim;
    struct timing t;
    struct file_parameters file;
    size_t max_runtime;
};

struct temporary {
    double *xphi, *yphi, *zphi; /* not written by the GPU path */
    double *grad, *lap;
    double *deltarho, *f;
    complex *deltarhoc, *fc, *phic;
};

struct k_grid {
    double *sq;
};

struct monitor {
    size_t calls_rhs;
    double total, integration, h5_write;
};

#define SUMMARY_VALUES (4)
#define NUMBER_CONSTRAINTS (4)

extern struct parameters pars;
extern double *field, *dfield;
extern double *rho, *pressure;
extern double rho_mean, pressure_mean;
extern struct output phi, dphi, psi, dpsi, rho_out;
extern struct output phi_smry, dphi_smry, psi_smry, dpsi_smry, rho_smry, p_smry;
extern struct output h1_smry, h2_smry;
extern struct output t_out, a_out;
extern struct output phi_ps, psi_ps, rho_ps;
extern struct output cstr, gw;
extern struct temporary tmp;
extern struct k_grid kvec;
extern struct monitor mon;

double get_wall_time();

#endif
