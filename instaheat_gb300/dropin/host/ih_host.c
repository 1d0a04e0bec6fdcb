/*
 * ih_host.c -- a standalone C99 host for the drop-in layer: it plays the part
 * of the reference's main.c, setup.c and io.c (globals, parameters, initial
 * state, the psi constraint solve, output buffers and save()), calling only
 * the reference-facing symbols of instaheat_dropin.h.
 *
 *   instaheat_host <initial-state.bin> <output.ihc> [final-state.bin]
 *
 * initial-state.bin holds Ntot doubles in the reference layout (phi, dphi,
 * psi, dpsi, h1, h2, dh1, dh2, a).  With INITIAL_CONDITIONS ==
 * IC_FROM_DAT_FILE_WITHOUT_PSI, psi and dpsi are solved from the constraints
 * as setup.c:825-868 does.  Outputs go to a flat container: "IHCONT01", then
 * records {u32 name length, name, u32 kind (0 parameter, 1 time-series
 * chunk), u64 rows, u64 dim, rows*dim doubles}; time-series chunks hold
 * WRITE_OUT_BUFFER_NUMBER slices (fewer in the last one), as the reference's
 * HDF5 datasets are extended.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include "main.h"
#include "io.h"
#include "instaheat_dropin.h"

struct parameters pars;
double *field, *dfield;
double *rho, *pressure;
double rho_mean, pressure_mean;
struct output phi, dphi, psi, dpsi, rho_out;
struct output phi_smry, dphi_smry, psi_smry, dpsi_smry, rho_smry, p_smry;
struct output h1_smry, h2_smry;
struct output t_out, a_out;
struct output phi_ps, psi_ps, rho_ps;
struct output cstr, gw;
struct temporary tmp;
struct k_grid kvec;
struct monitor mon;

static FILE *out_file = NULL;

double get_wall_time()
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

static void *xcalloc(size_t n, size_t size)
{
    void *p = calloc(n ? n : 1, size);
    if (!p) {
        fputs("Allocating memory failed.\n", stderr);
        exit(EXIT_FAILURE);
    }
    return p;
}

static void write_record(const char *name, unsigned kind, size_t rows, size_t dim,
                         const double *val)
{
    const unsigned len = (unsigned)strlen(name);
    const unsigned long long r = rows, d = dim;
    if (fwrite(&len, sizeof len, 1, out_file) != 1 || fwrite(name, 1, len, out_file) != len ||
        fwrite(&kind, sizeof kind, 1, out_file) != 1 || fwrite(&r, sizeof r, 1, out_file) != 1 ||
        fwrite(&d, sizeof d, 1, out_file) != 1 ||
        fwrite(val, sizeof *val, rows * dim, out_file) != rows * dim) {
        fputs("Writing the output container failed.\n", stderr);
        exit(EXIT_FAILURE);
    }
}

void h5_create_empty_by_path(const char *path)
{
    out_file = fopen(path, "wb");
    if (!out_file || fwrite("IHCONT01", 1, 8, out_file) != 8) {
        fprintf(stderr, "Cannot create %s\n", path);
        exit(EXIT_FAILURE);
    }
}

void h5_write_simple(const char *name, const double *val, const size_t N,
                     const H5D_layout_t layout)
{
    (void)layout;
    write_record(name, 0, 1, N, val);
}

void h5_write_followup()
{
    h5_write_simple(H5_FOLLOWUP_NAME, field, pars.Ntot, H5D_CONTIGUOUS);
}

static void alloc_output(struct output *o, size_t dim)
{
    o->dim = dim;
    o->buf = xcalloc(pars.file.buf_size * dim, sizeof(double));
    o->tmp = xcalloc(dim, sizeof(double));
}

static void free_output(struct output *o)
{
    free(o->buf);
    free(o->tmp);
    o->buf = o->tmp = NULL;
}

static void append_to_buffer(struct output *o)
{
    memcpy(o->buf + pars.file.index * o->dim, o->tmp, o->dim * sizeof(double));
}

static void flush_output(const char *name, const struct output *o, size_t rows)
{
    write_record(name, 1, rows, o->dim, o->buf);
}

/* every enabled time series, `rows` slices (io.c:361-441) */
static void write_all_buffers(size_t rows)
{
#ifdef OUTPUT_PHI
    flush_output(H5_PHI_NAME, &phi, rows);
#endif
#ifdef OUTPUT_DPHI
    flush_output(H5_DPHI_NAME, &dphi, rows);
#endif
#ifdef OUTPUT_PSI
    flush_output(H5_PSI_NAME, &psi, rows);
#endif
#ifdef OUTPUT_DPSI
    flush_output(H5_DPSI_NAME, &dpsi, rows);
#endif
#ifdef OUTPUT_RHO
    flush_output(H5_RHO_NAME, &rho_out, rows);
#endif
    flush_output(H5_TIME_NAME, &t_out, rows);
    flush_output(H5_A_NAME, &a_out, rows);
#ifdef OUTPUT_PHI_SMRY
    flush_output(H5_PHI_SMRY_NAME, &phi_smry, rows);
#endif
#ifdef OUTPUT_DPHI_SMRY
    flush_output(H5_DPHI_SMRY_NAME, &dphi_smry, rows);
#endif
#ifdef OUTPUT_PSI_SMRY
    flush_output(H5_PSI_SMRY_NAME, &psi_smry, rows);
#endif
#ifdef OUTPUT_DPSI_SMRY
    flush_output(H5_DPSI_SMRY_NAME, &dpsi_smry, rows);
#endif
#ifdef OUTPUT_RHO_SMRY
    flush_output(H5_RHO_SMRY_NAME, &rho_smry, rows);
#endif
#ifdef OUTPUT_PRESSURE_SMRY
    flush_output(H5_PRESSURE_SMRY_NAME, &p_smry, rows);
#endif
#ifdef OUTPUT_PHI_PS
    flush_output(H5_PHI_PS_NAME, &phi_ps, rows);
#endif
#ifdef OUTPUT_PSI_PS
    flush_output(H5_PSI_PS_NAME, &psi_ps, rows);
#endif
#ifdef OUTPUT_RHO_PS
    flush_output(H5_RHO_PS_NAME, &rho_ps, rows);
#endif
#ifdef OUTPUT_CONSTRAINTS
    flush_output(H5_CONSTRAINTS_NAME, &cstr, rows);
#endif
#ifdef ENABLE_GW
    flush_output(H5_GW_PS_NAME, &gw, rows);
#endif
}

void save()
{
    const size_t index = pars.file.index;
    a_out.tmp[0] = field[pars.Ntot - 1];
    append_to_buffer(&a_out);
    append_to_buffer(&t_out);
#ifdef OUTPUT_PHI_SMRY
    append_to_buffer(&phi_smry);
#endif
#ifdef OUTPUT_DPHI_SMRY
    append_to_buffer(&dphi_smry);
#endif
#ifdef OUTPUT_PSI_SMRY
    append_to_buffer(&psi_smry);
#endif
#ifdef OUTPUT_DPSI_SMRY
    append_to_buffer(&dpsi_smry);
#endif
#ifdef OUTPUT_RHO_SMRY
    append_to_buffer(&rho_smry);
#endif
#ifdef OUTPUT_PRESSURE_SMRY
    append_to_buffer(&p_smry);
#endif
#ifdef OUTPUT_PHI_PS
    append_to_buffer(&phi_ps);
#endif
#ifdef OUTPUT_PSI_PS
    append_to_buffer(&psi_ps);
#endif
#ifdef OUTPUT_RHO_PS
    append_to_buffer(&rho_ps);
#endif
#ifdef OUTPUT_CONSTRAINTS
    append_to_buffer(&cstr);
#endif
#ifdef ENABLE_GW
    append_to_buffer(&gw);
#endif
#ifdef LARGE_OUTPUT
    /* strided full fields (io.c:559-600) */
    const size_t Ny = pars.y.N, Nz = pars.z.N;
    const size_t os = index * pars.outN;
    for (size_t i = 0; i < pars.x.N; i += pars.x.stride) {
        const size_t osx = i * Ny * Nz;
        const size_t osxb = i * pars.y.outN * pars.z.outN / pars.x.stride;
        for (size_t j = 0; j < Ny; j += pars.y.stride) {
            const size_t osy = osx + j * Nz;
            const size_t osyb = osxb + j * pars.z.outN / pars.y.stride;
            for (size_t k = 0; k < Nz; k += pars.z.stride) {
                const size_t id = osy + k, idb = osyb + k / pars.z.stride;
#ifdef OUTPUT_PHI
                phi.buf[os + idb] = field[id];
#endif
#ifdef OUTPUT_DPHI
                dphi.buf[os + idb] = field[pars.N + id];
#endif
#ifdef OUTPUT_PSI
                psi.buf[os + idb] = field[2 * pars.N + id];
#endif
#ifdef OUTPUT_DPSI
                dpsi.buf[os + idb] = field[3 * pars.N + id];
#endif
#ifdef OUTPUT_RHO
                rho_out.buf[os + idb] = rho[id];
#endif
            }
        }
    }
#endif
    if (index == pars.file.buf_size - 1) {
        write_all_buffers(pars.file.buf_size);
        pars.file.index = 0;
    } else {
        pars.file.index += 1;
    }
}

void h5_close()
{
    if (pars.file.index != 0) {
        write_all_buffers(pars.file.index);
    }
    if (out_file) {
        fclose(out_file);
        out_file = NULL;
    }
}

static void init_pars(void)
{
    pars.x.N = GRIDPOINTS_X;
    pars.y.N = GRIDPOINTS_Y;
    pars.z.N = GRIDPOINTS_Z;
    pars.x.a = SPATIAL_LOWER_BOUND_X;
    pars.x.b = SPATIAL_UPPER_BOUND_X;
    pars.y.a = SPATIAL_LOWER_BOUND_Y;
    pars.y.b = SPATIAL_UPPER_BOUND_Y;
    pars.z.a = SPATIAL_LOWER_BOUND_Z;
    pars.z.b = SPATIAL_UPPER_BOUND_Z;
    pars.x.stride = STRIDE_X;
    pars.y.stride = STRIDE_Y;
    pars.z.stride = STRIDE_Z;
    struct grid_dimension *d[3] = {&pars.x, &pars.y, &pars.z};
    for (int i = 0; i < 3; ++i) {
        d[i]->k = TWOPI / (d[i]->b - d[i]->a);
        d[i]->k2 = d[i]->k * d[i]->k;
        d[i]->outN = (d[i]->N + d[i]->stride - 1) / d[i]->stride;
    }
    pars.x.M = pars.x.N;
    pars.y.M = pars.y.N;
    pars.z.M = pars.z.N / 2 + 1;
    pars.dim = 3;
    pars.N = pars.x.N * pars.y.N * pars.z.N;
    pars.M = pars.x.M * pars.y.M * pars.z.M;
    pars.Next = 2 * pars.M;
    pars.Ntot = 4 * pars.N + 4 * pars.Next + 1;
    pars.outN = pars.x.outN * pars.y.outN * pars.z.outN;
    pars.t.dt = DELTA_T;
    pars.t.t = INITIAL_TIME;
    pars.t.ti = INITIAL_TIME;
    pars.t.tf = FINAL_TIME;
    pars.t.Nt = (size_t)ceil((pars.t.tf - pars.t.ti) / pars.t.dt) + 1;
    pars.file.index = 0;
    pars.file.buf_size = WRITE_OUT_BUFFER_NUMBER;
    pars.file.skip = TIME_STEP_SKIPS;
    pars.max_runtime = MAX_RUNTIME;
}

/* k^2 on the half spectrum [x][y][z/2+1], with the Nyquist index kept */
static void init_ksq(void)
{
    const size_t nx = pars.x.N, ny = pars.y.N, mz = pars.z.M;
    kvec.sq = xcalloc(pars.M, sizeof(double));
    for (size_t i = 0; i < nx; ++i) {
        const double ki = (double)(i > nx / 2 ? nx - i : i);
        for (size_t j = 0; j < ny; ++j) {
            const double kj = (double)(j > ny / 2 ? ny - j : j);
            for (size_t k = 0; k < mz; ++k) {
                kvec.sq[(i * ny + j) * mz + k] = pars.z.k2 * (double)k * (double)k +
                                                 pars.x.k2 * ki * ki + pars.y.k2 * kj * kj;
            }
        }
    }
}

/* psi and dpsi from the Hamiltonian and momentum constraints, using the
 * drop-in's mk_rhs, mean, fft and ifft as setup.c:825-868 does */
static void initial_psi(void)
{
    const size_t N = pars.N;
    for (size_t i = 2 * N; i < 4 * N; ++i) {
        field[i] = 0.0;
    }
    evo_flags.output = 0;
    evo_flags.filter = 0;
    mk_rhs(pars.t.ti, field, dfield);
    const double a2 = field[pars.Ntot - 1] * field[pars.Ntot - 1];
    const double hubble = sqrt(rho_mean / 3.0);
    const double phi_mean = mean(field, N);
    const double dphi_mean = mean(field + N, N);
    const double ddphi_mean = mean(dfield + N, N);
    for (size_t i = 0; i < N; ++i) {
        tmp.deltarho[i] = field[N + i] - dphi_mean;
        tmp.f[i] = field[i] - phi_mean;
    }
    fft(tmp.deltarho, tmp.deltarhoc);
    fft(tmp.f, tmp.fc);
    for (size_t i = 1; i < pars.M; ++i) {
        tmp.phic[i] = (-dphi_mean * tmp.deltarhoc[i] + ddphi_mean * tmp.fc[i]) /
                      ((-dphi_mean * dphi_mean + 2.0 * kvec.sq[i] / a2) * (double)N);
    }
    tmp.phic[0] = 0.0;
    ifft(tmp.phic, field + 2 * N);
    for (size_t i = 0; i < N; ++i) {
        field[3 * N + i] = 0.5 * dphi_mean * tmp.f[i] - hubble * field[2 * N + i];
    }
}

static void allocate_all(void)
{
    field = xcalloc(pars.Ntot, sizeof(double));
    dfield = xcalloc(pars.Ntot, sizeof(double));
    rho = xcalloc(pars.N, sizeof(double));
    pressure = xcalloc(pars.N, sizeof(double));
    tmp.grad = xcalloc(pars.N, sizeof(double));
    tmp.lap = xcalloc(pars.N, sizeof(double));
    tmp.deltarho = xcalloc(pars.N, sizeof(double));
    tmp.f = xcalloc(pars.N, sizeof(double));
    tmp.deltarhoc = xcalloc(pars.M, sizeof(complex));
    tmp.fc = xcalloc(pars.M, sizeof(complex));
    tmp.phic = xcalloc(pars.M, sizeof(complex));
    const size_t bins = POWER_SPECTRUM_BINS;
    alloc_output(&t_out, 1);
    alloc_output(&a_out, 1);
#ifdef OUTPUT_PHI
    alloc_output(&phi, pars.outN);
#endif
#ifdef OUTPUT_DPHI
    alloc_output(&dphi, pars.outN);
#endif
#ifdef OUTPUT_PSI
    alloc_output(&psi, pars.outN);
#endif
#ifdef OUTPUT_DPSI
    alloc_output(&dpsi, pars.outN);
#endif
#ifdef OUTPUT_RHO
    alloc_output(&rho_out, pars.outN);
#endif
    alloc_output(&phi_smry, SUMMARY_VALUES);
    alloc_output(&dphi_smry, SUMMARY_VALUES);
    alloc_output(&psi_smry, SUMMARY_VALUES);
    alloc_output(&dpsi_smry, SUMMARY_VALUES);
    alloc_output(&rho_smry, SUMMARY_VALUES);
    alloc_output(&p_smry, SUMMARY_VALUES);
    alloc_output(&h1_smry, SUMMARY_VALUES);
    alloc_output(&h2_smry, SUMMARY_VALUES);
    alloc_output(&phi_ps, bins);
    alloc_output(&psi_ps, bins);
    alloc_output(&rho_ps, bins);
    alloc_output(&cstr, NUMBER_CONSTRAINTS);
    alloc_output(&gw, bins);
}

static void free_all(void)
{
    free(field);
    free(dfield);
    free(rho);
    free(pressure);
    free(tmp.grad);
    free(tmp.lap);
    free(tmp.deltarho);
    free(tmp.f);
    free(tmp.deltarhoc);
    free(tmp.fc);
    free(tmp.phic);
    free(kvec.sq);
    struct output *o[] = {&t_out, &a_out, &phi, &dphi, &psi, &dpsi, &rho_out,
                          &phi_smry, &dphi_smry, &psi_smry, &dpsi_smry, &rho_smry, &p_smry,
                          &h1_smry, &h2_smry, &phi_ps, &psi_ps, &rho_ps, &cstr, &gw};
    for (size_t i = 0; i < sizeof o / sizeof o[0]; ++i) {
        free_output(o[i]);
    }
}

static void write_parameters(void)
{
    double v[3];
    v[0] = MASS;
    h5_write_simple(H5_MASS_NAME, v, 1, H5D_COMPACT);
    v[0] = RELATIVE_TOLERANCE;
    v[1] = ABSOLUTE_TOLERANCE;
    h5_write_simple(H5_TOLERANCES_NAME, v, 2, H5D_COMPACT);
    v[0] = (double)pars.x.N;
    v[1] = (double)pars.y.N;
    v[2] = (double)pars.z.N;
    h5_write_simple(H5_GRIDPOINTS_INTERNAL_NAME, v, 3, H5D_COMPACT);
    v[0] = pars.x.a;
    v[1] = pars.x.b;
    h5_write_simple(H5_SPATIAL_BOUNDS_X_NAME, v, 2, H5D_COMPACT);
    v[0] = pars.y.a;
    v[1] = pars.y.b;
    h5_write_simple(H5_SPATIAL_BOUNDS_Y_NAME, v, 2, H5D_COMPACT);
    v[0] = pars.z.a;
    v[1] = pars.z.b;
    h5_write_simple(H5_SPATIAL_BOUNDS_Z_NAME, v, 2, H5D_COMPACT);
    v[0] = MAX_DT_HUBBLE_FRACTION;
    h5_write_simple(H5_MAX_DT_HUBBLE_FRACTION_NAME, v, 1, H5D_COMPACT);
#ifdef ENABLE_FFT_FILTER
    v[0] = 1.0;
#else
    v[0] = 0.0;
#endif
    h5_write_simple(H5_ENABLE_FILTER_NAME, v, 1, H5D_COMPACT);
#ifdef ENABLE_GW
    v[0] = 1.0;
#else
    v[0] = 0.0;
#endif
    h5_write_simple(H5_ENABLE_GW_NAME, v, 1, H5D_COMPACT);
}

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: %s initial-state.bin output.ihc [final-state.bin]\n", argv[0]);
        return EXIT_FAILURE;
    }
    mon.total = -get_wall_time();
    init_pars();
    init_ksq();
    allocate_all();
    FILE *in = fopen(argv[1], "rb");
    if (!in || fread(field, sizeof(double), pars.Ntot, in) != pars.Ntot) {
        fprintf(stderr, "Cannot read %zu doubles from %s\n", pars.Ntot, argv[1]);
        return EXIT_FAILURE;
    }
    fclose(in);
    h5_create_empty_by_path(argv[2]);
    write_parameters();
#if INITIAL_CONDITIONS == IC_FROM_DAT_FILE_WITHOUT_PSI
    initial_psi();
#endif
    t_out.tmp[0] = pars.t.ti;
    a_out.tmp[0] = field[pars.Ntot - 1];
#if INTEGRATION_METHOD == DOPRI853
    run_dopri853();
#elif INTEGRATION_METHOD == RK4
    run_rk4();
#else
#error "the drop-in layer provides the DOPRI853 and RK4 steppers"
#endif
    mon.total += get_wall_time();
    double v = (double)mon.calls_rhs;
    h5_write_simple(H5_COUNTER_RHS, &v, 1, H5D_COMPACT);
    h5_write_simple(H5_RUNTIME_TOTAL_NAME, &mon.total, 1, H5D_COMPACT);
    h5_close();
    if (argc > 3) {
        FILE *fo = fopen(argv[3], "wb");
        if (!fo || fwrite(field, sizeof(double), pars.Ntot, fo) != pars.Ntot) {
            fprintf(stderr, "Cannot write %s\n", argv[3]);
            return EXIT_FAILURE;
        }
        fclose(fo);
    }
    ih_dropin_release();
    free_all();
    return EXIT_SUCCESS;
}
