/*
 * ih_oracle.c -- CPU oracle: RHS, diagnostics, psi solve, DOPRI853, RK4, ICs.
 *
 * TEST INFRASTRUCTURE ONLY (see ih_oracle.h for the parity pin).  Each
 * function names the reference file:line it restates.  Complex arrays are
 * interleaved (re, im) doubles.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "ih_oracle_internal.h"

#define PI_D 3.141592653589793238462643383279
#define TWOPI_D 6.283185307179586476925286766559
#define MAXD(x, y) (((x) > (y)) ? (x) : (y))
#define MIND(x, y) (((x) > (y)) ? (y) : (x))

struct iho_ctx {
    iho_params p;
    size_t N, M, Next, Ntot;
    iho_fft3 F;
    /* k grid (setup.c:609-666) */
    double *kx, *ky, *kz, *kxf, *kyf, *kzf, *ksq, kmax;
    double *mask; /* filter (setup.c:710-754) */
    /* temporaries (main_template.h:254-271) */
    double *phic, *xphic, *yphic, *zphic, *fc, *psic, *deltarhoc, *cwork;
    double *xphi, *yphi, *zphi, *grad, *lap, *tf, *deltarho;
    double *rho, *pressure;
    double *s[6];
    double rho_mean, pressure_mean;
    unsigned long calls;
    /* DOPRI853 work vectors (dopri853.c:589-603) */
    double *k2, *k3, *k4, *k5, *k6, *k7, *k8, *k9, *k10, *ktmp, *yerr, *yerr2;
    double *field_new, *dfield_new;
};

void iho_sizes(int nx, int ny, int nz, size_t *N, size_t *M, size_t *Next,
               size_t *Ntot)
{
    /* setup.c:228, 263-271 (3D case) */
    size_t n = (size_t)nx * ny * nz;
    size_t m = (size_t)nx * ny * (nz / 2 + 1);
    if (N) *N = n;
    if (M) *M = m;
    if (Next) *Next = 2 * m;
    if (Ntot) *Ntot = 4 * n + 4 * (2 * m) + 1;
}

static double *dalloc(size_t n)
{
    double *p = calloc(n ? n : 1, sizeof(double));
    return p;
}

/* setup.c:609-666 */
static void build_kgrid(iho_ctx *c)
{
    const int Nx = c->p.nx, Ny = c->p.ny, Nz = c->p.nz;
    const int Mx = Nx, My = Ny, Mz = Nz / 2 + 1;
    const double kxu = TWOPI_D / c->p.lx, kyu = TWOPI_D / c->p.ly, kzu = TWOPI_D / c->p.lz;
    const double kx2 = kxu * kxu, ky2 = kyu * kyu, kz2 = kzu * kzu;
    for (int i = 0; i < Mx; ++i)
        for (int j = 0; j < My; ++j)
            for (int k = 0; k < Mz; ++k) {
                size_t id = ((size_t)i * My + j) * Mz + k;
                double q2 = kz2 * k * k;
                if (i > Nx / 2) {
                    c->kx[id] = kxu * (i - Nx);
                    c->kxf[id] = c->kx[id];
                    q2 += kx2 * (double)(Nx - i) * (Nx - i);
                } else if (2 * i == Nx) {
                    c->kx[id] = 0.0;
                    c->kxf[id] = kxu * i;
                    q2 += kx2 * (double)i * i;
                } else {
                    c->kx[id] = kxu * i;
                    c->kxf[id] = c->kx[id];
                    q2 += kx2 * (double)i * i;
                }
                if (j > Ny / 2) {
                    c->ky[id] = kyu * (j - Ny);
                    c->kyf[id] = c->ky[id];
                    q2 += ky2 * (double)(Ny - j) * (Ny - j);
                } else if (2 * j == Ny) {
                    c->ky[id] = 0.0;
                    c->kyf[id] = kyu * j;
                    q2 += ky2 * (double)j * j;
                } else {
                    c->ky[id] = kyu * j;
                    c->kyf[id] = c->ky[id];
                    q2 += ky2 * (double)j * j;
                }
                if (2 * k == Nz) {
                    c->kz[id] = 0.0;
                    c->kzf[id] = kzu * k;
                } else {
                    c->kz[id] = kzu * k;
                    c->kzf[id] = c->kz[id];
                }
                c->ksq[id] = q2;
            }
    double k2max = kx2 * (Nx / 2) * (Nx / 2) + ky2 * (Ny / 2) * (Ny / 2) +
                   kz2 * (Nz / 2) * (Nz / 2);
    c->kmax = sqrt(k2max);
}

/* setup.c:710-754: exp(-36 x^36), x = max_i |k_i| / k_i,max */
static void build_mask(iho_ctx *c)
{
    const double kxmax = (c->p.nx / 2) * (TWOPI_D / c->p.lx);
    const double kymax = (c->p.ny / 2) * (TWOPI_D / c->p.ly);
    const double kzmax = (c->p.nz / 2) * (TWOPI_D / c->p.lz);
    for (size_t i = 0; i < c->M; ++i) {
        double frac = fabs(c->kxf[i]) / kxmax;
        frac = MAXD(frac, fabs(c->kyf[i]) / kymax);
        frac = MAXD(frac, fabs(c->kzf[i]) / kzmax);
        c->mask[i] = exp(-36.0 * pow(frac, 36));
    }
}

iho_ctx *iho_create(const iho_params *p)
{
    if (p->nx < p->ny || p->ny < p->nz || p->nz < 2 || p->nz % 2) return NULL;
    iho_ctx *c = calloc(1, sizeof *c);
    c->p = *p;
#ifdef _OPENMP
    if (p->threads > 0) omp_set_num_threads(p->threads);
#endif
    iho_sizes(p->nx, p->ny, p->nz, &c->N, &c->M, &c->Next, &c->Ntot);
    if (iho_fft3_init(&c->F, p->nx, p->ny, p->nz)) {
        free(c);
        return NULL;
    }
    const size_t N = c->N, M = c->M, Ntot = c->Ntot;
    c->kx = dalloc(M); c->ky = dalloc(M); c->kz = dalloc(M);
    c->kxf = dalloc(M); c->kyf = dalloc(M); c->kzf = dalloc(M);
    c->ksq = dalloc(M); c->mask = dalloc(M);
    c->phic = dalloc(2 * M); c->xphic = dalloc(2 * M); c->yphic = dalloc(2 * M);
    c->zphic = dalloc(2 * M); c->fc = dalloc(2 * M); c->psic = dalloc(2 * M);
    c->deltarhoc = dalloc(2 * M); c->cwork = dalloc(2 * M);
    c->xphi = dalloc(N); c->yphi = dalloc(N); c->zphi = dalloc(N);
    c->grad = dalloc(N); c->lap = dalloc(N); c->tf = dalloc(N);
    c->deltarho = dalloc(N); c->rho = dalloc(N); c->pressure = dalloc(N);
    for (int j = 0; j < 6; ++j) c->s[j] = dalloc(2 * M);
    c->k2 = dalloc(Ntot); c->k3 = dalloc(Ntot); c->k4 = dalloc(Ntot);
    c->k5 = dalloc(Ntot); c->k6 = dalloc(Ntot); c->k7 = dalloc(Ntot);
    c->k8 = dalloc(Ntot); c->k9 = dalloc(Ntot); c->k10 = dalloc(Ntot);
    c->ktmp = dalloc(Ntot); c->yerr = dalloc(Ntot); c->yerr2 = dalloc(Ntot);
    c->field_new = dalloc(Ntot); c->dfield_new = dalloc(Ntot);
    build_kgrid(c);
    build_mask(c);
    return c;
}

void iho_destroy(iho_ctx *c)
{
    if (!c) return;
    iho_fft3_free(&c->F);
    double *arrs[] = {c->kx, c->ky, c->kz, c->kxf, c->kyf, c->kzf, c->ksq,
                      c->mask, c->phic, c->xphic, c->yphic, c->zphic, c->fc,
                      c->psic, c->deltarhoc, c->cwork, c->xphi, c->yphi,
                      c->zphi, c->grad, c->lap, c->tf, c->deltarho, c->rho,
                      c->pressure, c->k2, c->k3, c->k4, c->k5, c->k6, c->k7,
                      c->k8, c->k9, c->k10, c->ktmp, c->yerr, c->yerr2,
                      c->field_new, c->dfield_new};
    for (size_t i = 0; i < sizeof arrs / sizeof arrs[0]; ++i) free(arrs[i]);
    for (int j = 0; j < 6; ++j) free(c->s[j]);
    free(c);
}

void iho_kgrid(const iho_ctx *c, double *kx, double *ky, double *kz,
               double *kxf, double *kyf, double *kzf, double *ksq,
               double *kmax)
{
    size_t b = sizeof(double) * c->M;
    if (kx) memcpy(kx, c->kx, b);
    if (ky) memcpy(ky, c->ky, b);
    if (kz) memcpy(kz, c->kz, b);
    if (kxf) memcpy(kxf, c->kxf, b);
    if (kyf) memcpy(kyf, c->kyf, b);
    if (kzf) memcpy(kzf, c->kzf, b);
    if (ksq) memcpy(ksq, c->ksq, b);
    if (kmax) *kmax = c->kmax;
}

void iho_filter_mask(const iho_ctx *c, double *mask)
{
    memcpy(mask, c->mask, sizeof(double) * c->M);
}

/* toolbox.c:806-811 */
void iho_fft(iho_ctx *c, const double *in, double *out_c)
{
    iho_fft3_r2c(&c->F, in, out_c);
}

/* toolbox.c:822-827; the input is preserved (the oracle transforms a copy) */
void iho_ifft(iho_ctx *c, const double *in_c, double *out)
{
    memcpy(c->cwork, in_c, sizeof(double) * 2 * c->M);
    iho_fft3_c2r(&c->F, c->cwork, out);
}

double iho_mean(const double *f, size_t n)
{
    /* toolbox.c:726-734 */
    double m = 0.0;
    #pragma omp parallel for reduction(+: m)
    for (size_t i = 0; i < n; ++i) m += f[i];
    return m / n;
}

double iho_variance(double mean, const double *f, size_t n)
{
    /* toolbox.c:744-754 (corrected two-pass, N-1) */
    double s1 = 0.0, s2 = 0.0;
    #pragma omp parallel for reduction(+: s1, s2)
    for (size_t i = 0; i < n; ++i) {
        double d = f[i] - mean;
        s1 += d * d;
        s2 += d;
    }
    return (s1 - s2 * s2 / n) / (n - 1);
}

/* toolbox.c:596-626: in *= filter; out = c2r(in / N) */
static void capply_filter(iho_ctx *c, double *in, double *out)
{
    const size_t M = c->M;
    const double Nd = (double)c->N;
    #pragma omp parallel for
    for (size_t i = 0; i < M; ++i) {
        in[2 * i] *= c->mask[i];
        in[2 * i + 1] *= c->mask[i];
        c->deltarhoc[2 * i] = in[2 * i] / Nd;
        c->deltarhoc[2 * i + 1] = in[2 * i + 1] / Nd;
    }
    iho_ifft(c, c->deltarhoc, out);
}

static void apply_filter(iho_ctx *c, double *f)
{
    iho_fft(c, f, c->fc);
    capply_filter(c, c->fc, f);
}

/* toolbox.c:160-186 */
static void mk_ffts_and_filter(iho_ctx *c, double *f, int filter, int output)
{
    const size_t N = c->N, M = c->M;
    iho_fft(c, f, c->phic);
    if (c->p.filter) {
        if (filter == 1) {
            iho_fft(c, f + 2 * N, c->psic);
            capply_filter(c, c->phic, f);
            capply_filter(c, c->psic, f + 2 * N);
            apply_filter(c, f + N);
            apply_filter(c, f + 3 * N);
        }
    } else if (output == 1) {
        iho_fft(c, f + 2 * N, c->psic);
    }
    if (output == 1) {
        #pragma omp parallel for
        for (size_t i = 0; i < M; ++i) {
            c->fc[2 * i] = -c->psic[2 * i] * c->ksq[i] / (double)N;
            c->fc[2 * i + 1] = -c->psic[2 * i + 1] * c->ksq[i] / (double)N;
        }
        iho_ifft(c, c->fc, c->tf);
    }
}

/* toolbox.c:129-149 and 196-208 */
static void mk_gradient_squared_and_laplacian(iho_ctx *c, double *f, int filter,
                                              int output)
{
    const size_t M = c->M, N = c->N;
    mk_ffts_and_filter(c, f, filter, output);
    #pragma omp parallel for
    for (size_t i = 0; i < M; ++i) {
        double pr = c->phic[2 * i] / (double)N, pi = c->phic[2 * i + 1] / (double)N;
        /* pre * I * k = (-pi k, pr k) */
        c->xphic[2 * i] = -pi * c->kx[i];
        c->xphic[2 * i + 1] = pr * c->kx[i];
        c->yphic[2 * i] = -pi * c->ky[i];
        c->yphic[2 * i + 1] = pr * c->ky[i];
        c->zphic[2 * i] = -pi * c->kz[i];
        c->zphic[2 * i + 1] = pr * c->kz[i];
        c->fc[2 * i] = -pr * c->ksq[i];
        c->fc[2 * i + 1] = -pi * c->ksq[i];
    }
    iho_ifft(c, c->xphic, c->xphi);
    iho_ifft(c, c->yphic, c->yphi);
    iho_ifft(c, c->zphic, c->zphi);
    iho_ifft(c, c->fc, c->lap);
    #pragma omp parallel for
    for (size_t i = 0; i < N; ++i) {
        c->grad[i] = c->xphi[i] * c->xphi[i];
        c->grad[i] += c->yphi[i] * c->yphi[i];
        c->grad[i] += c->zphi[i] * c->zphi[i];
    }
}

static inline double potential(const iho_ctx *c, double f)
{
    return c->p.mass * c->p.mass * f * f / 2.0; /* toolbox.c:493-497 */
}

static inline double potential_prime(const iho_ctx *c, double f)
{
    return c->p.mass * c->p.mass * f; /* toolbox.c:506-510 */
}

/* toolbox.c:225-243 */
static void mk_rho_and_p(iho_ctx *c, const double *f)
{
    const size_t N = c->N;
    const double a2 = f[c->Ntot - 1] * f[c->Ntot - 1];
    double rm = 0.0, pm = 0.0;
    #pragma omp parallel for reduction(+: rm, pm)
    for (size_t i = 0; i < N; ++i) {
        double dph = f[N + i], ps = f[2 * N + i];
        double t1 = (0.5 - ps) * dph * dph;
        double t2 = (0.5 + ps) * c->grad[i] / a2;
        c->rho[i] = t1 + t2 + potential(c, f[i]);
        c->pressure[i] = t1 - t2 / 3.0 - potential(c, f[i]);
        pm += c->pressure[i];
        rm += c->rho[i];
    }
    c->rho_mean = rm / N;
    c->pressure_mean = pm / N;
}

/* toolbox.c:567-582 */
static void mk_power_spectrum(const iho_ctx *c, const double *in, double *out)
{
    const int bins = c->p.bins;
    for (int i = 0; i < bins; ++i) out[i] = 0.0;
    for (size_t i = 1; i < c->M; ++i) {
        double p2 = in[2 * i] * in[2 * i] + in[2 * i + 1] * in[2 * i + 1];
        if (fabs(c->kz[i]) > DBL_EPSILON) p2 *= 2.0;
        size_t idx = (int)trunc(bins * sqrt(c->ksq[i]) / c->kmax - 1.0e-14);
        if (idx >= (size_t)bins) idx = bins - 1;  /* |k| = k_max: see mk_gw_spectrum */
        out[idx] += p2 / c->N;
    }
}

/* toolbox.c:676-690 */
static void mean_var_min_max(const double *f, double *smry, size_t N)
{
    double m = 0.0, mn = f[0], mx = f[0];
    #pragma omp parallel for reduction(+: m) reduction(max: mx) reduction(min: mn)
    for (size_t i = 0; i < N; ++i) {
        m += f[i];
        mn = MIND(mn, f[i]);
        mx = MAXD(mx, f[i]);
    }
    smry[0] = m / N;
    smry[1] = iho_variance(smry[0], f, N);
    smry[2] = mn;
    smry[3] = mx;
}

/* toolbox.c:524-551 */
static void mk_constraints(iho_ctx *c, const double *f, double *cstr)
{
    const size_t N = c->N;
    const double a2 = f[c->Ntot - 1] * f[c->Ntot - 1];
    const double hubble = sqrt(c->rho_mean / 3.0);
    const double h3 = 3.0 * hubble;
    const double phi_mean = iho_mean(f, N);
    const double dphi_mean = iho_mean(f + N, N);
    double hl2 = 0.0, hmax = 0.0, ml2 = 0.0, mmax = 0.0;
    #pragma omp parallel for reduction(max: hmax, mmax) reduction(+: hl2, ml2)
    for (size_t i = 0; i < N; ++i) {
        double t1 = hubble * f[2 * N + i] + f[3 * N + i];
        double ham = c->tf[i] / a2 - h3 * t1 - 0.5 * (c->rho[i] - c->rho_mean);
        double mom = t1 - 0.5 * dphi_mean * (f[i] - phi_mean);
        hl2 += ham * ham;
        ml2 += mom * mom;
        hmax = MAXD(hmax, fabs(ham));
        mmax = MAXD(mmax, fabs(mom));
    }
    cstr[0] = hl2 / N;
    cstr[1] = hmax;
    cstr[2] = ml2 / N;
    cstr[3] = mmax;
}

/* toolbox.c:435-484 */
static void mk_gw_spectrum(const iho_ctx *c, const double *f, double *gw)
{
    const size_t N = c->N, Next = c->Next;
    const size_t Ndh1 = 4 * N + 2 * Next, Ndh2 = Ndh1 + Next;
    const double hubble = sqrt(c->rho_mean / 3.0);
    const double rat = pow(0.01, 1.0 / 3.0);
    const double fac = PI_D * rat / (3.0 * hubble * hubble * c->p.lx * c->p.ly * c->p.lz);
    const int bins = c->p.bins;
    for (int i = 0; i < bins; ++i) gw[i] = 0.0;
    for (size_t i = 1; i < c->M; ++i) {
        double kx = c->kxf[i], ky = c->kyf[i], kz = c->kzf[i];
        double kx2 = kx * kx, ky2 = ky * ky, kz2 = kz * kz;
        double k2 = c->ksq[i], k = sqrt(k2);
        double d1r = f[Ndh1 + 2 * i], d2r = f[Ndh2 + 2 * i];
        double d1i = f[Ndh1 + 2 * i + 1], d2i = f[Ndh2 + 2 * i + 1];
        double pw;
        if (fabs(kz) > DBL_EPSILON) {
            pw = 2.0 * k2 / (kz2 * (ky2 + kz2)) *
                 ((kx2 + kz2) * (d1r * d1r + d1i * d1i) +
                  2.0 * kx * ky * (d1r * d2r + d1i * d2i) +
                  (ky2 + kz2) * (d2r * d2r + d2i * d2i));
        } else if (fabs(ky) > DBL_EPSILON) {
            pw = 2.0 * (kx2 + ky2) / (ky2 * ky2) *
                 ((kx2 + ky2) * (d1r * d1r + d1i * d1i) + ky2 * (d2r * d2r + d2i * d2i));
        } else {
            pw = 2.0 * (d1r * d1r + d1i * d1i + d2r * d2r + d2i * d2i);
        }
        if (fabs(c->kz[i]) > DBL_EPSILON) pw *= 2.0;
        size_t idx = (int)trunc(bins * k / c->kmax - 1.0e-14);
        /* The - 1e-14 of toolbox.c:479 puts |k| = k_max (the grid corner) into
         * the last bin; where bins * k / k_max rounds to exactly `bins` (e.g.
         * 512^3 with 256 bins) the subtraction is lost to rounding and
         * toolbox.c writes one past its array.  The corner mode is kept in
         * the last bin here, as the offset intends (the GPU does the same). */
        if (idx >= (size_t)bins) idx = bins - 1;
        gw[idx] += fac * k2 * k * pw;
    }
    for (int i = 0; i < bins; ++i) gw[i] /= N;
}

/* toolbox.c:251-270, 634-663 */
static void output_all(iho_ctx *c, const double *f, iho_output *out,
                       const double *smry_src)
{
    const size_t N = c->N;
    if (!out) return;
    if (out->phi_ps) mk_power_spectrum(c, c->phic, out->phi_ps);
    if (out->psi_ps) mk_power_spectrum(c, c->psic, out->psi_ps);
    if (out->rho_ps) {
        iho_fft(c, c->rho, c->fc);
        mk_power_spectrum(c, c->fc, out->rho_ps);
    }
    mk_constraints(c, f, out->cstr);
    /* mk_summary() reads the global `field`, which during the post-step RHS
       of dopri853.c:291 still holds the previous step's state */
    const double *g = smry_src ? smry_src : f;
    mean_var_min_max(g, out->smry[0], N);
    mean_var_min_max(g + N, out->smry[1], N);
    mean_var_min_max(g + 2 * N, out->smry[2], N);
    mean_var_min_max(g + 3 * N, out->smry[3], N);
    mean_var_min_max(c->rho, out->smry[4], N);
    mean_var_min_max(c->pressure, out->smry[5], N);
    if (c->p.gw && out->gw) mk_gw_spectrum(c, f, out->gw);
}

/* toolbox.c:282-299 */
static void update_phi_psi(iho_ctx *c, const double *f, double *result)
{
    const size_t N = c->N, N2 = 2 * N, N3 = 3 * N;
    const double a2 = f[c->Ntot - 1] * f[c->Ntot - 1];
    const double hubble = sqrt(c->rho_mean / 3.0);
    const double h3 = 3.0 * hubble;
    const double pm = c->pressure_mean;
    #pragma omp parallel for
    for (size_t i = 0; i < N; ++i) {
        double dph = f[N + i], ps = f[N2 + i], dps = f[N3 + i];
        result[i] = dph;
        result[N + i] = (1.0 + 4.0 * ps) * c->lap[i] / a2 - (h3 - 4.0 * dps) * dph -
                        (1.0 + 2.0 * ps) * potential_prime(c, f[i]);
        result[N2 + i] = dps;
        result[N3 + i] = 0.5 * c->pressure[i] + (ps - 0.5) * pm - 4.0 * hubble * dps;
    }
}

/* toolbox.c:410-424 */
static void mk_gw_sources(iho_ctx *c)
{
    double *t1[] = {c->xphi, c->xphi, c->xphi, c->yphi, c->yphi, c->zphi};
    double *t2[] = {c->xphi, c->yphi, c->zphi, c->yphi, c->zphi, c->zphi};
    const size_t N = c->N;
    for (int j = 0; j < 6; ++j) {
        #pragma omp parallel for
        for (size_t i = 0; i < N; ++i) c->deltarho[i] = t1[j][i] * t2[j][i];
        iho_fft(c, c->deltarho, c->s[j]);
    }
}

/* complex helpers on interleaved pairs */
typedef struct { double r, i; } cpx;
static inline cpx cl(const double *a, size_t i) { cpx z = {a[2 * i], a[2 * i + 1]}; return z; }
static inline cpx cadd(cpx a, cpx b) { cpx z = {a.r + b.r, a.i + b.i}; return z; }
static inline cpx csub(cpx a, cpx b) { cpx z = {a.r - b.r, a.i - b.i}; return z; }
static inline cpx cscl(double s, cpx a) { cpx z = {s * a.r, s * a.i}; return z; }

/* toolbox.c:363-397 */
static void mk_gw_sources_tt(iho_ctx *c)
{
    mk_gw_sources(c);
    double **s = c->s;
    #pragma omp parallel for
    for (size_t i = 1; i < c->M; ++i) {
        double kx = c->kxf[i], ky = c->kyf[i], kz = c->kzf[i];
        double ksq = c->ksq[i];
        double fx = kx / ksq, fy = ky / ksq, fz = kz / ksq;
        cpx s0 = cl(s[0], i), s1v = cl(s[1], i), s2v = cl(s[2], i);
        cpx s3 = cl(s[3], i), s4 = cl(s[4], i), s5 = cl(s[5], i);
        cpx t1 = cadd(cadd(cadd(cscl(kx * fx, s0), cscl(ky * fy, s3)), cscl(kz * fz, s5)),
                      cscl(2.0, cadd(cadd(cscl(kx * fy, s1v), cscl(kx * fz, s2v)),
                                     cscl(ky * fz, s4))));
        cpx t2 = cadd(cadd(s0, s3), s5);
        cpx S1 = cadd(t1, t2), S2 = csub(t1, t2);
        cpx n0, n1;
        if (fabs(kz) > DBL_EPSILON) {
            cpx k1 = cadd(cadd(cscl(kx, s0), cscl(ky, s1v)), cscl(kz, s2v));
            cpx k2 = cadd(cadd(cscl(kx, s1v), cscl(ky, s3)), cscl(kz, s4));
            n0 = cadd(csub(s0, cscl(2.0 * fx, k1)), cscl(0.5, cadd(cscl(fx * kx, S1), S2)));
            n1 = cadd(csub(csub(s1v, cscl(fx, k2)), cscl(fy, k1)), cscl(0.5 * fx * ky, S1));
        } else if (fabs(ky) > DBL_EPSILON) {
            cpx k1 = cadd(cadd(cscl(kx, s0), cscl(ky, s1v)), cscl(kz, s2v));
            cpx k3 = cadd(cadd(cscl(kx, s2v), cscl(ky, s4)), cscl(kz, s5));
            n0 = cadd(csub(s0, cscl(2.0 * fx, k1)), cscl(0.5, cadd(cscl(fx * kx, S1), S2)));
            n1 = cadd(csub(csub(s2v, cscl(fx, k3)), cscl(fz, k1)), cscl(0.5 * fx * kz, S1));
        } else {
            cpx k2 = cadd(cadd(cscl(kx, s1v), cscl(ky, s3)), cscl(kz, s4));
            cpx k3 = cadd(cadd(cscl(kx, s2v), cscl(ky, s4)), cscl(kz, s5));
            n0 = cadd(csub(s3, cscl(2.0 * fy, k2)), cscl(0.5, cadd(cscl(fy * ky, S1), S2)));
            n1 = cadd(csub(csub(s4, cscl(fy, k3)), cscl(fz, k2)), cscl(0.5 * fy * kz, S1));
        }
        s[0][2 * i] = n0.r; s[0][2 * i + 1] = n0.i;
        s[1][2 * i] = n1.r; s[1][2 * i + 1] = n1.i;
    }
    s[0][0] = s[0][1] = 0.0;
    s[1][0] = s[1][1] = 0.0;
}

/* toolbox.c:311-346 */
static void update_h(iho_ctx *c, const double *f, double *result)
{
    const size_t N = c->N, Next = c->Next, Nh1 = 4 * N, Nh2 = Nh1 + Next;
    const size_t Ndh1 = Nh2 + Next, Ndh2 = Ndh1 + Next;
    const double a2 = f[c->Ntot - 1] * f[c->Ntot - 1];
    const double hubble = sqrt(c->rho_mean / 3.0);
    const double h3 = 3.0 * hubble;
    #pragma omp parallel for
    for (size_t i = 0; i < 2 * Next; ++i) result[Nh1 + i] = f[Ndh1 + i];
    mk_gw_sources_tt(c);
    double **s = c->s;
    #pragma omp parallel for
    for (size_t i = 0; i < c->M; ++i) {
        size_t i1 = 2 * i, i2 = i1 + 1;
        double tm = -(2.0 * c->pressure_mean + c->ksq[i] / a2);
        result[Ndh1 + i1] = tm * f[Nh1 + i1] - h3 * f[Ndh1 + i1] + 2.0 * s[0][i1] / a2;
        result[Ndh1 + i2] = tm * f[Nh1 + i2] - h3 * f[Ndh1 + i2] + 2.0 * s[0][i2] / a2;
        result[Ndh2 + i1] = tm * f[Nh2 + i1] - h3 * f[Ndh2 + i1] + 2.0 * s[1][i1] / a2;
        result[Ndh2 + i2] = tm * f[Nh2 + i2] - h3 * f[Ndh2 + i2] + 2.0 * s[1][i2] / a2;
    }
}

static void mk_rhs_impl(iho_ctx *c, double t, double *f, double *result,
                        int filter, int output, iho_output *out,
                        const double *smry_src)
{
    (void)t;
    c->calls += 1;
    mk_gradient_squared_and_laplacian(c, f, filter, output);
    mk_rho_and_p(c, f);
    if (output == 1) output_all(c, f, out, smry_src);
    update_phi_psi(c, f, result);
    if (c->p.gw) update_h(c, f, result);
    result[c->Ntot - 1] = f[c->Ntot - 1] * sqrt(c->rho_mean / 3.0);
}

/* toolbox.c:75-88 */
void iho_mk_rhs(iho_ctx *c, double t, double *f, double *result, int filter,
                int output, iho_output *out)
{
    mk_rhs_impl(c, t, f, result, filter, output, out, NULL);
}

double iho_rho_mean(const iho_ctx *c) { return c->rho_mean; }
double iho_pressure_mean(const iho_ctx *c) { return c->pressure_mean; }
const double *iho_rho(const iho_ctx *c) { return c->rho; }
const double *iho_pressure(const iho_ctx *c) { return c->pressure; }
const double *iho_lap(const iho_ctx *c) { return c->lap; }
const double *iho_grad2(const iho_ctx *c) { return c->grad; }
unsigned long iho_calls_rhs(const iho_ctx *c) { return c->calls; }

/* setup.c:825-903 */
void iho_initial_psi(iho_ctx *c, double *f, double t)
{
    const size_t N = c->N, M = c->M;
    for (size_t i = 2 * N; i < 4 * N; ++i) f[i] = 0.0;
    double *df = c->dfield_new;
    mk_rhs_impl(c, t, f, df, 0, 0, NULL, NULL);
    const double a2 = f[c->Ntot - 1] * f[c->Ntot - 1];
    const double hubble = sqrt(c->rho_mean / 3.0);
    const double phi_mean = iho_mean(f, N);
    const double dphi_mean = iho_mean(f + N, N);
    const double ddphi_mean = iho_mean(df + N, N);
    #pragma omp parallel for
    for (size_t i = 0; i < N; ++i) {
        c->deltarho[i] = f[N + i] - dphi_mean;
        c->tf[i] = f[i] - phi_mean;
    }
    iho_fft(c, c->deltarho, c->deltarhoc);
    iho_fft(c, c->tf, c->fc);
    #pragma omp parallel for
    for (size_t i = 1; i < M; ++i) {
        double den = (-dphi_mean * dphi_mean + 2.0 * c->ksq[i] / a2) * N;
        c->phic[2 * i] = (-dphi_mean * c->deltarhoc[2 * i] + ddphi_mean * c->fc[2 * i]) / den;
        c->phic[2 * i + 1] =
            (-dphi_mean * c->deltarhoc[2 * i + 1] + ddphi_mean * c->fc[2 * i + 1]) / den;
    }
    c->phic[0] = c->phic[1] = 0.0;
    iho_ifft(c, c->phic, f + 2 * N);
    #pragma omp parallel for
    for (size_t i = 0; i < N; ++i) f[3 * N + i] = 0.5 * dphi_mean * c->tf[i] - hubble * f[2 * N + i];
}

/* ------------------------------------------------------------------------ */
/* DOPRI853.  Coefficients of the Dormand-Prince 8(5,3) pair as published by  */
/* Hairer, Norsett & Wanner (code DOP853), in the form the reference uses     */
/* (src/dopri853_constants.c:11-176, Numerical Recipes' Dopr853 layout).      */
/* Stages are numbered 1..12; A[i][j] is a_{i+1, j+1}.                        */
/* ------------------------------------------------------------------------ */
static const double DP_C[12] = {
    0.0,
    0.526001519587677318785587544488e-01,
    0.789002279381515978178381316732e-01,
    0.118350341907227396726757197510e+00,
    0.281649658092772603273242802490e+00,
    0.333333333333333333333333333333e+00,
    0.25e+00,
    0.307692307692307692307692307692e+00,
    0.651282051282051282051282051282e+00,
    0.6e+00,
    0.857142857142857142857142857142e+00,
    1.0};

static double DP_A[12][12];
static double DP_B[12], DP_E3[12], DP_BHH[3];
/* dense output (dopri853_constants.c:23-25, 98-173; declared but unused by
   the reference's stepper): the inputs of stages 14-16 over stages 1..16
   (stage 13 = f(field_new)) and the weights d4..d7 of the continuous
   extension's last four coefficient vectors */
static double DP_AD[3][16], DP_D[4][16];
static int dp_ready = 0;

static void dp_init(void)
{
    if (dp_ready) return;
    memset(DP_A, 0, sizeof DP_A);
    memset(DP_B, 0, sizeof DP_B);
    memset(DP_E3, 0, sizeof DP_E3);
    double (*A)[12] = DP_A;
    A[1][0] = 5.26001519587677318785587544488e-2;
    A[2][0] = 1.97250569845378994544595329183e-2;
    A[2][1] = 5.91751709536136983633785987549e-2;
    A[3][0] = 2.95875854768068491816892993775e-2;
    A[3][2] = 8.87627564304205475450678981324e-2;
    A[4][0] = 2.41365134159266685502369798665e-1;
    A[4][2] = -8.84549479328286085344864962717e-1;
    A[4][3] = 9.24834003261792003115737966543e-1;
    A[5][0] = 3.7037037037037037037037037037e-2;
    A[5][3] = 1.70828608729473871279604482173e-1;
    A[5][4] = 1.25467687566822425016691814123e-1;
    A[6][0] = 3.7109375e-2;
    A[6][3] = 1.70252211019544039314978060272e-1;
    A[6][4] = 6.02165389804559606850219397283e-2;
    A[6][5] = -1.7578125e-2;
    A[7][0] = 3.70920001185047927108779319836e-2;
    A[7][3] = 1.70383925712239993810214054705e-1;
    A[7][4] = 1.07262030446373284651809199168e-1;
    A[7][5] = -1.53194377486244017527936158236e-2;
    A[7][6] = 8.27378916381402288758473766002e-3;
    A[8][0] = 6.24110958716075717114429577812e-1;
    A[8][3] = -3.36089262944694129406857109825e0;
    A[8][4] = -8.68219346841726006818189891453e-1;
    A[8][5] = 2.75920996994467083049415600797e1;
    A[8][6] = 2.01540675504778934086186788979e1;
    A[8][7] = -4.34898841810699588477366255144e1;
    A[9][0] = 4.77662536438264365890433908527e-1;
    A[9][3] = -2.48811461997166764192642586468e0;
    A[9][4] = -5.90290826836842996371446475743e-1;
    A[9][5] = 2.12300514481811942347288949897e1;
    A[9][6] = 1.52792336328824235832596922938e1;
    A[9][7] = -3.32882109689848629194453265587e1;
    A[9][8] = -2.03312017085086261358222928593e-2;
    A[10][0] = -9.3714243008598732571704021658e-1;
    A[10][3] = 5.18637242884406370830023853209e0;
    A[10][4] = 1.09143734899672957818500254654e0;
    A[10][5] = -8.14978701074692612513997267357e0;
    A[10][6] = -1.85200656599969598641566180701e1;
    A[10][7] = 2.27394870993505042818970056734e1;
    A[10][8] = 2.49360555267965238987089396762e0;
    A[10][9] = -3.0467644718982195003823669022e0;
    A[11][0] = 2.27331014751653820792359768449e0;
    A[11][3] = -1.05344954667372501984066689879e1;
    A[11][4] = -2.00087205822486249909675718444e0;
    A[11][5] = -1.79589318631187989172765950534e1;
    A[11][6] = 2.79488845294199600508499808837e1;
    A[11][7] = -2.85899827713502369474065508674e0;
    A[11][8] = -8.87285693353062954433549289258e0;
    A[11][9] = 1.23605671757943030647266201528e1;
    A[11][10] = 6.43392746015763530355970484046e-1;
    DP_B[0] = 5.42937341165687622380535766363e-2;
    DP_B[5] = 4.45031289275240888144113950566e0;
    DP_B[6] = 1.89151789931450038304281599044e0;
    DP_B[7] = -5.8012039600105847814672114227e0;
    DP_B[8] = 3.1116436695781989440891606237e-1;
    DP_B[9] = -1.52160949662516078556178806805e-1;
    DP_B[10] = 2.01365400804030348374776537501e-1;
    DP_B[11] = 4.47106157277725905176885569043e-2;
    DP_BHH[0] = 0.244094488188976377952755905512e+00; /* stage 1 */
    DP_BHH[1] = 0.733846688281611857341361741547e+00; /* stage 9 */
    DP_BHH[2] = 0.220588235294117647058823529412e-01; /* stage 12 */
    DP_E3[0] = 0.1312004499419488073250102996e-01;
    DP_E3[5] = -0.1225156446376204440720569753e+01;
    DP_E3[6] = -0.4957589496572501915214079952e+00;
    DP_E3[7] = 0.1664377182454986536961530415e+01;
    DP_E3[8] = -0.3503288487499736816886487290e+00;
    DP_E3[9] = 0.3341791187130174790297318841e+00;
    DP_E3[10] = 0.8192320648511571246570742613e-01;
    DP_E3[11] = -0.2235530786388629525884427845e-01;
    memset(DP_AD, 0, sizeof DP_AD);
    memset(DP_D, 0, sizeof DP_D);
    double (*AD)[16] = DP_AD, (*DD)[16] = DP_D;
    AD[0][0] = 5.61675022830479523392909219681e-2;
    AD[0][6] = 2.53500210216624811088794765333e-1;
    AD[0][7] = -2.46239037470802489917441475441e-1;
    AD[0][8] = -1.24191423263816360469010140626e-1;
    AD[0][9] = 1.5329179827876569731206322685e-1;
    AD[0][10] = 8.20105229563468988491666602057e-3;
    AD[0][11] = 7.56789766054569976138603589584e-3;
    AD[0][12] = -8.298e-3;
    AD[1][0] = 3.18346481635021405060768473261e-2;
    AD[1][5] = 2.83009096723667755288322961402e-2;
    AD[1][6] = 5.35419883074385676223797384372e-2;
    AD[1][7] = -5.49237485713909884646569340306e-2;
    AD[1][10] = -1.08347328697249322858509316994e-4;
    AD[1][11] = 3.82571090835658412954920192323e-4;
    AD[1][12] = -3.40465008687404560802977114492e-4;
    AD[1][13] = 1.41312443674632500278074618366e-1;
    AD[2][0] = -4.28896301583791923408573538692e-1;
    AD[2][5] = -4.69762141536116384314449447206e0;
    AD[2][6] = 7.68342119606259904184240953878e0;
    AD[2][7] = 4.06898981839711007970213554331e0;
    AD[2][8] = 3.56727187455281109270669543021e-1;
    AD[2][12] = -1.39902416515901462129418009734e-3;
    AD[2][13] = 2.9475147891527723389556272149e0;
    AD[2][14] = -9.15095847217987001081870187138e0;
    DD[0][0] = -0.84289382761090128651353491142e+01;
    DD[0][5] = 0.56671495351937776962531783590e+00;
    DD[0][6] = -0.30689499459498916912797304727e+01;
    DD[0][7] = 0.23846676565120698287728149680e+01;
    DD[0][8] = 0.21170345824450282767155149946e+01;
    DD[0][9] = -0.87139158377797299206789907490e+00;
    DD[0][10] = 0.22404374302607882758541771650e+01;
    DD[0][11] = 0.63157877876946881815570249290e+00;
    DD[0][12] = -0.88990336451333310820698117400e-01;
    DD[0][13] = 0.18148505520854727256656404962e+02;
    DD[0][14] = -0.91946323924783554000451984436e+01;
    DD[0][15] = -0.44360363875948939664310572000e+01;
    DD[1][0] = 0.10427508642579134603413151009e+02;
    DD[1][5] = 0.24228349177525818288430175319e+03;
    DD[1][6] = 0.16520045171727028198505394887e+03;
    DD[1][7] = -0.37454675472269020279518312152e+03;
    DD[1][8] = -0.22113666853125306036270938578e+02;
    DD[1][9] = 0.77334326684722638389603898808e+01;
    DD[1][10] = -0.30674084731089398182061213626e+02;
    DD[1][11] = -0.93321305264302278729567221706e+01;
    DD[1][12] = 0.15697238121770843886131091075e+02;
    DD[1][13] = -0.31139403219565177677282850411e+02;
    DD[1][14] = -0.93529243588444783865713862664e+01;
    DD[1][15] = 0.35816841486394083752465898540e+02;
    DD[2][0] = 0.19985053242002433820987653617e+02;
    DD[2][5] = -0.38703730874935176555105901742e+03;
    DD[2][6] = -0.18917813819516756882830838328e+03;
    DD[2][7] = 0.52780815920542364900561016686e+03;
    DD[2][8] = -0.11573902539959630126141871134e+02;
    DD[2][9] = 0.68812326946963000169666922661e+01;
    DD[2][10] = -0.10006050966910838403183860980e+01;
    DD[2][11] = 0.77771377980534432092869265740e+00;
    DD[2][12] = -0.27782057523535084065932004339e+01;
    DD[2][13] = -0.60196695231264120758267380846e+02;
    DD[2][14] = 0.84320405506677161018159903784e+02;
    DD[2][15] = 0.11992291136182789328035130030e+02;
    DD[3][0] = -0.25693933462703749003312586129e+02;
    DD[3][5] = -0.15418974869023643374053993627e+03;
    DD[3][6] = -0.23152937917604549567536039109e+03;
    DD[3][7] = 0.35763911791061412378285349910e+03;
    DD[3][8] = 0.93405324183624310003907691704e+02;
    DD[3][9] = -0.37458323136451633156875139351e+02;
    DD[3][10] = 0.10409964950896230045147246184e+03;
    DD[3][11] = 0.29840293426660503123344363579e+02;
    DD[3][12] = -0.43533456590011143754432175058e+02;
    DD[3][13] = 0.96324553959188282948394950600e+02;
    DD[3][14] = -0.39177261675615439165231486172e+02;
    DD[3][15] = -0.14972683625798562581422125276e+03;
    dp_ready = 1;
}

void iho_dopri853_dense_tableau(double *ad, double *d)
{
    dp_init();
    if (ad) memcpy(ad, DP_AD, sizeof DP_AD);
    if (d) memcpy(d, DP_D, sizeof DP_D);
}

void iho_dopri853_tableau(double *c, double *a, double *b, double *bhh,
                          double *er)
{
    dp_init();
    if (c) memcpy(c, DP_C, sizeof DP_C);
    if (a) memcpy(a, DP_A, sizeof DP_A);
    if (b) memcpy(b, DP_B, sizeof DP_B);
    if (bhh) memcpy(bhh, DP_BHH, sizeof DP_BHH);
    if (er) memcpy(er, DP_E3, sizeof DP_E3);
}

/* dopri853.c:331-458.  ks[0] = dfield (stage 1), ks[j] = stage j+1. */
static void try_step(iho_ctx *c, const double *field, const double *dfield,
                     double t, double dt)
{
    dp_init();
    const size_t Ntot = c->Ntot;
    /* stage buffers in the reference's reuse pattern: stage 11 -> k2,
       stage 12 -> k3 (dopri853.c:423, 436) */
    double *kb[12] = {(double *)dfield, c->k2, c->k3, c->k4, c->k5, c->k6,
                      c->k7, c->k8, c->k9, c->k10, NULL, NULL};
    for (int s = 1; s < 12; ++s) {
        double *dst = (s == 10) ? c->k2 : (s == 11) ? c->k3 : kb[s];
        #pragma omp parallel for
        for (size_t i = 0; i < Ntot; ++i) {
            double acc = 0.0;
            for (int j = 0; j < s; ++j)
                if (DP_A[s][j] != 0.0) acc += DP_A[s][j] * kb[j][i];
            c->ktmp[i] = field[i] + dt * acc;
        }
        double ts = (s == 11) ? t + dt : t + DP_C[s] * dt;
        mk_rhs_impl(c, ts, c->ktmp, dst, 0, 0, NULL, NULL);
        if (s == 10) kb[10] = c->k2;
        else if (s == 11) kb[11] = c->k3;
    }
    /* NOTE: after stage 11 the k2 buffer holds stage 11; stage 2 is no longer
       needed (a_{12,2} = a_{11,2} = 0 and b_2 = 0).  Same for stage 3. */
    #pragma omp parallel for
    for (size_t i = 0; i < Ntot; ++i) {
        double k4 = DP_B[0] * dfield[i] + DP_B[5] * kb[5][i] + DP_B[6] * kb[6][i] +
                    DP_B[7] * kb[7][i] + DP_B[8] * kb[8][i] + DP_B[9] * kb[9][i] +
                    DP_B[10] * kb[10][i] + DP_B[11] * kb[11][i];
        c->field_new[i] = field[i] + dt * k4;
        c->yerr[i] = k4 - DP_BHH[0] * dfield[i] - DP_BHH[1] * kb[8][i] - DP_BHH[2] * kb[11][i];
        c->yerr2[i] = DP_E3[0] * dfield[i] + DP_E3[5] * kb[5][i] + DP_E3[6] * kb[6][i] +
                      DP_E3[7] * kb[7][i] + DP_E3[8] * kb[8][i] + DP_E3[9] * kb[9][i] +
                      DP_E3[10] * kb[10][i] + DP_E3[11] * kb[11][i];
    }
}

/* dopri853.c:469-486 */
static double dp_error(iho_ctx *c, const iho_dopri_cfg *cfg, const double *field,
                       double dt)
{
    double err = 0.0, err2 = 0.0;
    const size_t Ntot = c->Ntot;
    #pragma omp parallel for reduction(+: err, err2)
    for (size_t i = 0; i < Ntot; ++i) {
        double sk = cfg->atol + cfg->rtol * MAXD(fabs(field[i]), fabs(c->field_new[i]));
        double q = c->yerr[i] / sk;
        err2 += q * q;
        q = c->yerr2[i] / sk;
        err += q * q;
    }
    double deno = err + 0.01 * err2;
    if (deno <= 0.0) deno = 1.0;
    return dt * err * sqrt(1.0 / (Ntot * deno));
}

/* dopri853.c:505-540 */
static int dp_success(iho_ctx *c, const iho_dopri_cfg *cfg, iho_dopri_state *st,
                      double err, double *dt)
{
    const double alpha = 1.0 / 8.0 - cfg->beta * 0.2;
    double scale;
    if (err <= 1.0) {
        if (err == 0.0) {
            scale = cfg->maxscale;
        } else {
            scale = cfg->safe * pow(err, -alpha) * pow(st->err_old, cfg->beta);
            if (scale < cfg->minscale) scale = cfg->minscale;
            if (scale > cfg->maxscale) scale = cfg->maxscale;
        }
        if (st->reject) st->dt_next = (*dt) * MIND(scale, 1.0);
        else st->dt_next = (*dt) * scale;
        if (cfg->max_dt_hubble_fraction > 0.0) {
            const double minstep = cfg->max_dt_hubble_fraction * sqrt(3.0 / c->rho_mean);
            if (st->dt_next > minstep) st->dt_next = minstep;
        }
        st->err_old = MAXD(err, 1.0e-4);
        st->reject = 0;
        return 1;
    }
    scale = MAXD(cfg->safe * pow(err, -alpha), cfg->minscale);
    (*dt) *= scale;
    st->reject = 1;
    return 0;
}

/* dopri853.c:172-198 + prepare_and_save_timeslice (toolbox.c:96-104) */
void iho_dopri853_init(iho_ctx *c, const iho_dopri_cfg *cfg,
                       iho_dopri_state *st, double *field, double *dfield,
                       double t0, double dt0)
{
    (void)cfg;
    memset(st, 0, sizeof *st);
    st->t = t0;
    st->dt = dt0;
    st->dt_next = dt0;
    st->err_old = 1.0e-4;
    mk_rhs_impl(c, t0, field, dfield, 1, 0, NULL, NULL);
}

/* The continuous extension of the accepted step (Hairer, Norsett & Wanner,
   the DOP853 dense output; coefficients dopri853_constants.c:23-25, 98-173):
   stages 14-16 from y = field, the stages of the try (stage 1 = dfield, 6..10
   in k6..k10, 11 in k2, 12 in k3) and stage 13 = dfield_new = f(field_new),
   then per element
     r1 = y, r2 = field_new - y, r3 = dt k1 - r2, r4 = r2 - dt k13 - r3,
     r(5+i) = dt sum_j d(4+i)j k_j,
     y(theta) = r1 + theta (r2 + s (r3 + theta (r4 + s (r5 + theta (r6
                + s (r7 + theta r8)))))),  s = 1 - theta.
   field_new is the state after the post-step RHS (filtered in place when the
   filter is on).  Stages 14-16 go to the buffers of stages 4, 5 and yerr. */
static void dense_output(iho_ctx *c, const double *field, const double *dfield,
                         double t, double dt, int n, const double *theta,
                         double *out)
{
    dp_init();
    const size_t Ntot = c->Ntot;
    const double *kb[16] = {dfield, NULL, NULL, NULL, NULL, c->k6, c->k7,
                            c->k8, c->k9, c->k10, c->k2, c->k3,
                            c->dfield_new, c->k4, c->k5, c->yerr};
    for (int r = 0; r < 3; ++r) {
        #pragma omp parallel for
        for (size_t i = 0; i < Ntot; ++i) {
            double acc = 0.0;
            for (int j = 0; j < 13 + r; ++j)
                if (DP_AD[r][j] != 0.0) acc += DP_AD[r][j] * kb[j][i];
            c->ktmp[i] = field[i] + dt * acc;
        }
        mk_rhs_impl(c, t, c->ktmp, (double *)kb[13 + r], 0, 0, NULL, NULL);
    }
    for (int q = 0; q < n; ++q) {
        const double th = theta[q], s1 = 1.0 - th;
        double *o = out + (size_t)q * Ntot;
        #pragma omp parallel for
        for (size_t i = 0; i < Ntot; ++i) {
            double d[4];
            for (int r = 0; r < 4; ++r) {
                double acc = 0.0;
                for (int j = 0; j < 16; ++j)
                    if (DP_D[r][j] != 0.0) acc += DP_D[r][j] * kb[j][i];
                d[r] = dt * acc;
            }
            const double r1 = field[i], r2 = c->field_new[i] - field[i];
            const double r3 = dt * dfield[i] - r2;
            const double r4 = r2 - dt * c->dfield_new[i] - r3;
            o[i] = r1 + th * (r2 + s1 * (r3 + th * (r4 + s1 * (d[0] + th * (d[1] +
                   s1 * (d[2] + th * d[3]))))));
        }
    }
}

static int dopri853_step_impl(iho_ctx *c, const iho_dopri_cfg *cfg,
                              iho_dopri_state *st, double *field, double *dfield,
                              double dt_try, iho_output *out, int n_dense,
                              const double *theta, double *dense_out)
{
    double dt = dt_try;
    for (;;) {
        try_step(c, field, dfield, st->t, dt);
        st->tries += 1;
        double err = dp_error(c, cfg, field, dt);
        st->last_err = err;
        if (dp_success(c, cfg, st, err, &dt)) break;
        if (fabs(dt) <= fabs(st->t) * DBL_EPSILON) return 1;
    }
    mk_rhs_impl(c, st->t + dt, c->field_new, c->dfield_new, 1, out ? 1 : 0, out,
                field);
    if (n_dense > 0) dense_output(c, field, dfield, st->t, dt, n_dense, theta, dense_out);
    memcpy(field, c->field_new, sizeof(double) * c->Ntot);
    memcpy(dfield, c->dfield_new, sizeof(double) * c->Ntot);
    st->t += (st->dt_did = dt);
    return 0;
}

/* dopri853.c:271-311 */
int iho_dopri853_step(iho_ctx *c, const iho_dopri_cfg *cfg,
                      iho_dopri_state *st, double *field, double *dfield,
                      double dt_try, iho_output *out)
{
    return dopri853_step_impl(c, cfg, st, field, dfield, dt_try, out, 0, NULL, NULL);
}

int iho_dopri853_step_dense(iho_ctx *c, const iho_dopri_cfg *cfg,
                            iho_dopri_state *st, double *field, double *dfield,
                            double dt_try, int n, const double *theta,
                            double *dense_out)
{
    return dopri853_step_impl(c, cfg, st, field, dfield, dt_try, NULL, n, theta,
                              dense_out);
}

/* dopri853.c:112-158 (without I/O) */
long iho_dopri853_run(iho_ctx *c, const iho_dopri_cfg *cfg,
                      iho_dopri_state *st, double *field, double *dfield,
                      double tf, long max_steps, double *log, long log_cap)
{
    long accepted = 0;
    for (st->n_stp = 0;; ++st->n_stp) {
        if (st->t + st->dt * 1.0001 > tf) st->dt = tf - st->t;
        long tries0 = st->tries;
        if (iho_dopri853_step(c, cfg, st, field, dfield, st->dt, NULL)) break;
        ++accepted;
        if (st->dt_did == st->dt) ++st->n_ok;
        else ++st->n_bad;
        if (log && st->n_stp < log_cap) {
            log[4 * st->n_stp] = st->t;
            log[4 * st->n_stp + 1] = st->dt_did;
            log[4 * st->n_stp + 2] = st->last_err;
            log[4 * st->n_stp + 3] = (double)(st->tries - tries0);
        }
        if (st->t >= tf) break;
        if (st->n_stp + 1 >= max_steps) break;
        if (fabs(st->dt_next) <= cfg->dt_min) break;
        st->dt = st->dt_next;
    }
    return accepted;
}

/* rk4.c:63-102 (filter on stage 1, no output) */
void iho_rk4_step(iho_ctx *c, double *field, double t, double dt)
{
    const size_t Ntot = c->Ntot;
    double *k1 = c->k2, *k2 = c->k3, *k3 = c->k4, *k4 = c->k5, *tk = c->ktmp;
    mk_rhs_impl(c, t, field, k1, 1, 0, NULL, NULL);
    #pragma omp parallel for
    for (size_t i = 0; i < Ntot; ++i) tk[i] = field[i] + dt * k1[i] / 2.0;
    mk_rhs_impl(c, t + dt / 2.0, tk, k2, 0, 0, NULL, NULL);
    #pragma omp parallel for
    for (size_t i = 0; i < Ntot; ++i) tk[i] = field[i] + dt * k2[i] / 2.0;
    mk_rhs_impl(c, t + dt / 2.0, tk, k3, 0, 0, NULL, NULL);
    #pragma omp parallel for
    for (size_t i = 0; i < Ntot; ++i) tk[i] = field[i] + dt * k3[i];
    mk_rhs_impl(c, t + dt, tk, k4, 0, 0, NULL, NULL);
    #pragma omp parallel for
    for (size_t i = 0; i < Ntot; ++i)
        field[i] += dt * (k1[i] + 2.0 * k2[i] + 2.0 * k3[i] + k4[i]) / 6.0;
}

/* ------------------------------------------------------------------------ */
/* Seeded fluctuation ICs.  Counter-based generator: SplitMix64 finaliser of  */
/* (mix(seed) xor counter), 53-bit uniforms in (0,1), Box-Muller.             */
/* ------------------------------------------------------------------------ */
static uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double uniform01(uint64_t key, uint64_t ctr)
{
    uint64_t r = mix64(key ^ mix64(ctr));
    return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

static void normal_pair(uint64_t key, uint64_t idx, double *g1, double *g2)
{
    double u1 = uniform01(key, 2 * idx), u2 = uniform01(key, 2 * idx + 1);
    double r = sqrt(-2.0 * log(u1));
    *g1 = r * cos(TWOPI_D * u2);
    *g2 = r * sin(TWOPI_D * u2);
}

void iho_ic_fluctuations(iho_ctx *c, double *f, unsigned long long seed,
                         double phi0, double dphi0, double a0, double amp,
                         double kcut)
{
    const int Nx = c->p.nx, Ny = c->p.ny, Nz = c->p.nz, Mz = Nz / 2 + 1;
    const size_t N = c->N, M = c->M;
    const double vol = c->p.lx * c->p.ly * c->p.lz;
    const double m2 = c->p.mass * c->p.mass;
    const uint64_t key = mix64((uint64_t)seed);
    double *cphi = c->xphic, *cdphi = c->yphic;
    #pragma omp parallel for
    for (size_t id = 0; id < M; ++id) {
        int k = (int)(id % Mz);
        int j = (int)((id / Mz) % Ny);
        int i = (int)(id / ((size_t)Mz * Ny));
        double re = 0.0, im = 0.0, omega = 0.0;
        double ksq = c->ksq[id];
        if (id != 0 && ksq <= kcut * kcut) {
            omega = sqrt(ksq + m2);
            double sigma = amp / sqrt(2.0 * omega * vol);
            int self_plane = (k == 0) || (2 * k == Nz);
            int pi = (Nx - i) % Nx, pj = (Ny - j) % Ny;
            size_t pid = ((size_t)pi * Ny + pj) * Mz + k;
            double g1, g2;
            if (self_plane && pid == id) {
                normal_pair(key, id, &g1, &g2);
                re = sigma * g1;
                im = 0.0;
            } else if (self_plane && pid < id) {
                normal_pair(key, pid, &g1, &g2);
                re = sigma * g1 / sqrt(2.0);
                im = -sigma * g2 / sqrt(2.0);
            } else {
                normal_pair(key, id, &g1, &g2);
                re = sigma * g1 / sqrt(2.0);
                im = sigma * g2 / sqrt(2.0);
            }
        }
        cphi[2 * id] = re;
        cphi[2 * id + 1] = im;
        /* delta dphi_k = -i omega delta phi_k */
        cdphi[2 * id] = omega * im;
        cdphi[2 * id + 1] = -omega * re;
    }
    iho_ifft(c, cphi, f);
    iho_ifft(c, cdphi, f + N);
    #pragma omp parallel for
    for (size_t i = 0; i < N; ++i) {
        f[i] += phi0;
        f[N + i] += dphi0;
        f[2 * N + i] = 0.0;
        f[3 * N + i] = 0.0;
    }
    for (size_t i = 4 * N; i < c->Ntot - 1; ++i) f[i] = 0.0;
    f[c->Ntot - 1] = a0;
}
