/*
 * io.h (standalone host) -- the output calls the drop-in layer makes
 * (save, h5_write_simple, h5_write_followup; the reference's io.h:73-99) and
 * the dataset names of the reference's output file (io.h:13-71).
 *
 * The standalone host writes the same datasets -- names, per-slice
 * dimensions, time-series chunks of WRITE_OUT_BUFFER_NUMBER slices, scalar
 * parameter datasets -- into a flat container (ih_host.c) instead of HDF5,
 * which is not available here; instaheat_gb300/dropin/container.py reads it.
 */
#ifndef __FILEHANDLING__
#define __FILEHANDLING__

#include <stddef.h>

#define H5_PHI_NAME                     ("phi")
#define H5_DPHI_NAME                    ("dphi")
#define H5_PSI_NAME                     ("psi")
#define H5_DPSI_NAME                    ("dpsi")
#define H5_RHO_NAME                     ("rho")
#define H5_PHI_PS_NAME                  ("phi_power_spectrum")
#define H5_PSI_PS_NAME                  ("psi_power_spectrum")
#define H5_RHO_PS_NAME                  ("rho_power_spectrum")
#define H5_GW_PS_NAME                   ("gravitational_wave_spectrum")
#define H5_TIME_NAME                    ("time")
#define H5_A_NAME                       ("a")
#define H5_PHI_SMRY_NAME                ("phi_summary")
#define H5_DPHI_SMRY_NAME               ("dphi_summary")
#define H5_PSI_SMRY_NAME                ("psi_summary")
#define H5_DPSI_SMRY_NAME               ("dpsi_summary")
#define H5_RHO_SMRY_NAME                ("rho_summary")
#define H5_PRESSURE_SMRY_NAME           ("pressure_summary")
#define H5_H1_SMRY_NAME                 ("h1_summary")
#define H5_H2_SMRY_NAME                 ("h2_summary")
#define H5_CONSTRAINTS_NAME             ("constraints")
#define H5_MASS_NAME                    ("mass")
#define H5_TOLERANCES_NAME              ("tolerances")
#define H5_GRIDPOINTS_INTERNAL_NAME     ("gridpoints_internal")
#define H5_SPATIAL_BOUNDS_X_NAME        ("spatial_bounds_x")
#define H5_SPATIAL_BOUNDS_Y_NAME        ("spatial_bounds_y")
#define H5_SPATIAL_BOUNDS_Z_NAME        ("spatial_bounds_z")
#define H5_RUNTIME_TOTAL_NAME           ("runtime_total")
#define H5_RUNTIME_STEPPER_NAME         ("runtime_stepper")
#define H5_COUNTER_RHS                  ("calls_rhs")
#define H5_STEPS_TOTAL_NAME             ("steps_total")
#define H5_STEPS_OK_NAME                ("steps_ok")
#define H5_STEPS_BAD_NAME               ("steps_bad")
#define H5_MAX_DT_HUBBLE_FRACTION_NAME  ("max_dt_hubble_fraction")
#define H5_ENABLE_FILTER_NAME           ("filter")
#define H5_ENABLE_GW_NAME               ("gravitational_waves")
#define H5_FOLLOWUP_NAME                ("followup")

/* dataset storage kinds (HDF5's H5D_layout_t values the reference passes) */
typedef enum { H5D_COMPACT = 0, H5D_CONTIGUOUS = 1, H5D_CHUNKED = 2 } H5D_layout_t;

void h5_create_empty_by_path(const char *path);
void h5_write_simple(const char *name, const double *val, const size_t N,
                     const H5D_layout_t layout);
void save();
void h5_close();
void h5_write_followup();

#endif
