/*
 * ih_oracle_fft.c -- FP64 3D real FFTs for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see ih_oracle.h).  The reference calls FFTW3
 * (src/toolbox.c:806-827, plans src/setup.c:524-554, FFTW_ESTIMATE by default
 * in src/parameters.sh:31), a third-party library that is not vendored in the
 * reference and not installed here.  This file restates the transforms FFTW
 * computes, with FFTW's conventions: r2c is the unnormalised DFT with
 * exp(-2 pi i jk/n), c2r the unnormalised inverse with exp(+2 pi i jk/n) over
 * the Hermitian-completed spectrum, half spectrum laid out [nx][ny][nz/2+1].
 *
 * Algorithm: self-sorting (Stockham) mixed-radix 2/3/4/5 transforms along
 * each axis, applied to batches of B pencils stored pencil-index innermost so
 * the butterflies vectorise; the real z-axis uses the half-length complex
 * transform with the standard even/odd post-processing.  Twiddles are taken
 * from sin/cos of exactly reduced angles.  OpenMP parallelises over batches.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "ih_oracle_internal.h"

#define PB 8 /* pencils per batch */

static const double TWO_PI = 6.283185307179586476925286766559;

static void unit_root(long num, long den, int sign, double *re, double *im)
{
    /* exp(sign * 2 pi i num/den) with num reduced mod den first */
    long r = num % den;
    if (r < 0) r += den;
    double ang = TWO_PI * (double)r / (double)den;
    *re = cos(ang);
    *im = sign * sin(ang);
}

int iho_cplan_init(iho_cplan *p, int n)
{
    memset(p, 0, sizeof *p);
    p->n = n;
    int len = n;
    while (len > 1) {
        int r;
        if (len % 4 == 0) r = 4;
        else if (len % 2 == 0) r = 2;
        else if (len % 3 == 0) r = 3;
        else if (len % 5 == 0) r = 5;
        else return -1; /* unsupported prime factor */
        p->radix[p->nst++] = r;
        len /= r;
    }
    /* twiddles per stage: for stage with current length L and radix r,
       m = L/r, stored w(pp, t) = exp(+2 pi i pp t / L), pp < m, 1 <= t < r;
       the imaginary part takes the transform's sign when used */
    len = n;
    for (int s = 0; s < p->nst; ++s) {
        int r = p->radix[s], m = len / r;
        p->tw[s] = malloc(sizeof(double) * 2 * (size_t)m * (r - 1) + 16);
        for (int pp = 0; pp < m; ++pp)
            for (int t = 1; t < r; ++t) {
                double re, im;
                unit_root((long)pp * t, len, +1, &re, &im);
                p->tw[s][2 * ((size_t)pp * (r - 1) + t - 1)] = re;
                p->tw[s][2 * ((size_t)pp * (r - 1) + t - 1) + 1] = im;
            }
        len = m;
    }
    return 0;
}

void iho_cplan_free(iho_cplan *p)
{
    for (int s = 0; s < p->nst; ++s) free(p->tw[s]);
    memset(p, 0, sizeof *p);
}

/* Batched complex transform in place on x (length n, batch b innermost:
 * element (idx, q) at 2*(idx*b + q)).  work has the same size.  sign=-1
 * forward, +1 backward.  Unnormalised. */
void iho_cfft_batch(const iho_cplan *p, double *x, double *work, int b,
                    int sign)
{
    const int n = p->n;
    double *src = x, *dst = work;
    int len = n, s = 1; /* current sub-length and stride (in pencils units) */
    for (int st = 0; st < p->nst; ++st) {
        const int r = p->radix[st], m = len / r;
        const double *tw = p->tw[st];
        for (int pp = 0; pp < m; ++pp) {
            for (int q = 0; q < s; ++q) {
                /* inputs: src[q + s*(pp + t*m)], t < r ; each is a batch of b */
                const double *a[5];
                double *o[5];
                for (int t = 0; t < r; ++t) {
                    a[t] = src + 2 * (size_t)b * (q + (size_t)s * (pp + (size_t)t * m));
                    o[t] = dst + 2 * (size_t)b * (q + (size_t)s * ((size_t)r * pp + t));
                }
                double wr[5] = {1, 1, 1, 1, 1}, wi[5] = {0, 0, 0, 0, 0};
                for (int t = 1; t < r; ++t) {
                    wr[t] = tw[2 * ((size_t)pp * (r - 1) + t - 1)];
                    wi[t] = sign * tw[2 * ((size_t)pp * (r - 1) + t - 1) + 1];
                }
                if (r == 2) {
                    for (int v = 0; v < b; ++v) {
                        double ar = a[0][2 * v], ai = a[0][2 * v + 1];
                        double br = a[1][2 * v], bi = a[1][2 * v + 1];
                        double dr = ar - br, di = ai - bi;
                        o[0][2 * v] = ar + br;
                        o[0][2 * v + 1] = ai + bi;
                        o[1][2 * v] = dr * wr[1] - di * wi[1];
                        o[1][2 * v + 1] = dr * wi[1] + di * wr[1];
                    }
                } else if (r == 4) {
                    for (int v = 0; v < b; ++v) {
                        double x0r = a[0][2 * v], x0i = a[0][2 * v + 1];
                        double x1r = a[1][2 * v], x1i = a[1][2 * v + 1];
                        double x2r = a[2][2 * v], x2i = a[2][2 * v + 1];
                        double x3r = a[3][2 * v], x3i = a[3][2 * v + 1];
                        double s02r = x0r + x2r, s02i = x0i + x2i;
                        double d02r = x0r - x2r, d02i = x0i - x2i;
                        double s13r = x1r + x3r, s13i = x1i + x3i;
                        double d13r = x1r - x3r, d13i = x1i - x3i;
                        /* multiply d13 by sign*i: (sign*i)(dr + i di) = -sign di + i sign dr */
                        double jr = -sign * d13i, ji = sign * d13r;
                        double y0r = s02r + s13r, y0i = s02i + s13i;
                        double y2r = s02r - s13r, y2i = s02i - s13i;
                        double y1r = d02r + jr, y1i = d02i + ji;
                        double y3r = d02r - jr, y3i = d02i - ji;
                        o[0][2 * v] = y0r;
                        o[0][2 * v + 1] = y0i;
                        o[1][2 * v] = y1r * wr[1] - y1i * wi[1];
                        o[1][2 * v + 1] = y1r * wi[1] + y1i * wr[1];
                        o[2][2 * v] = y2r * wr[2] - y2i * wi[2];
                        o[2][2 * v + 1] = y2r * wi[2] + y2i * wr[2];
                        o[3][2 * v] = y3r * wr[3] - y3i * wi[3];
                        o[3][2 * v + 1] = y3r * wi[3] + y3i * wr[3];
                    }
                } else {
                    /* generic small-radix DFT (3, 5): y_t = sum_u a_u e^{sign 2 pi i ut/r} */
                    double cr[5][5], ci[5][5];
                    for (int t = 0; t < r; ++t)
                        for (int u = 0; u < r; ++u)
                            unit_root((long)t * u, r, sign, &cr[t][u], &ci[t][u]);
                    for (int v = 0; v < b; ++v) {
                        for (int t = 0; t < r; ++t) {
                            double yr = 0.0, yi = 0.0;
                            for (int u = 0; u < r; ++u) {
                                double xr = a[u][2 * v], xi = a[u][2 * v + 1];
                                yr += xr * cr[t][u] - xi * ci[t][u];
                                yi += xr * ci[t][u] + xi * cr[t][u];
                            }
                            o[t][2 * v] = yr * wr[t] - yi * wi[t];
                            o[t][2 * v + 1] = yr * wi[t] + yi * wr[t];
                        }
                    }
                }
            }
        }
        double *tmp = src;
        src = dst;
        dst = tmp;
        len = m;
        s *= r;
    }
    if (src != x) memcpy(x, src, sizeof(double) * 2 * (size_t)n * b);
}

/* ---- real z-axis helpers ---- */

/* rows: b real rows of length nz starting at in + row0*nz (consecutive rows);
 * writes nz/2+1 complex per row to out (row stride mz complex). */
static void z_r2c_batch(const iho_fft3 *F, const double *in, double *out, int b,
                        double *buf, double *work)
{
    const int nz = F->nz, h = nz / 2, mz = h + 1;
    for (int j = 0; j < h; ++j)
        for (int v = 0; v < b; ++v) {
            buf[2 * ((size_t)j * b + v)] = in[(size_t)v * nz + 2 * j];
            buf[2 * ((size_t)j * b + v) + 1] = in[(size_t)v * nz + 2 * j + 1];
        }
    iho_cfft_batch(&F->pz, buf, work, b, -1);
    for (int v = 0; v < b; ++v) {
        double *o = out + 2 * (size_t)v * mz;
        for (int k = 0; k <= h; ++k) {
            int k1 = k % h, k2 = (h - k) % h;
            double zr = buf[2 * ((size_t)k1 * b + v)], zi = buf[2 * ((size_t)k1 * b + v) + 1];
            double cr = buf[2 * ((size_t)k2 * b + v)], ci = -buf[2 * ((size_t)k2 * b + v) + 1];
            double er = 0.5 * (zr + cr), ei = 0.5 * (zi + ci);
            /* O = (Z - conj Z_{h-k}) / (2i) */
            double dr = 0.5 * (zr - cr), di = 0.5 * (zi - ci);
            double orr = di, oi = -dr;
            double wr = F->wz[2 * k], wi = F->wz[2 * k + 1]; /* exp(-2 pi i k/nz) */
            o[2 * k] = er + (orr * wr - oi * wi);
            o[2 * k + 1] = ei + (orr * wi + oi * wr);
        }
    }
}

static void z_c2r_batch(const iho_fft3 *F, const double *in, double *out, int b,
                        double *buf, double *work)
{
    const int nz = F->nz, h = nz / 2, mz = h + 1;
    for (int v = 0; v < b; ++v) {
        const double *x = in + 2 * (size_t)v * mz;
        for (int k = 0; k < h; ++k) {
            double xr = x[2 * k], xi = x[2 * k + 1];
            double cr = x[2 * (h - k)], ci = -x[2 * (h - k) + 1];
            double er = xr + cr, ei = xi + ci;
            double dr = xr - cr, di = xi - ci;
            /* O = D * exp(+2 pi i k/nz) */
            double wr = F->wz[2 * k], wi = -F->wz[2 * k + 1];
            double orr = dr * wr - di * wi, oi = dr * wi + di * wr;
            /* Z = E + i O */
            buf[2 * ((size_t)k * b + v)] = er - oi;
            buf[2 * ((size_t)k * b + v) + 1] = ei + orr;
        }
    }
    iho_cfft_batch(&F->pz, buf, work, b, +1);
    for (int j = 0; j < h; ++j)
        for (int v = 0; v < b; ++v) {
            out[(size_t)v * nz + 2 * j] = buf[2 * ((size_t)j * b + v)];
            out[(size_t)v * nz + 2 * j + 1] = buf[2 * ((size_t)j * b + v) + 1];
        }
}

int iho_fft3_init(iho_fft3 *F, int nx, int ny, int nz)
{
    memset(F, 0, sizeof *F);
    F->nx = nx;
    F->ny = ny;
    F->nz = nz;
    if (nz < 2 || nz % 2) return -1;
    if (iho_cplan_init(&F->px, nx) || iho_cplan_init(&F->py, ny) ||
        iho_cplan_init(&F->pz, nz / 2))
        return -1;
    F->wz = malloc(sizeof(double) * 2 * (nz / 2 + 1));
    for (int k = 0; k <= nz / 2; ++k)
        unit_root(k, nz, -1, &F->wz[2 * k], &F->wz[2 * k + 1]);
    F->maxn = nx > ny ? nx : ny;
    if (nz > F->maxn) F->maxn = nz;
    return 0;
}

void iho_fft3_free(iho_fft3 *F)
{
    iho_cplan_free(&F->px);
    iho_cplan_free(&F->py);
    iho_cplan_free(&F->pz);
    free(F->wz);
    memset(F, 0, sizeof *F);
}

/* Transform along y then x (or x then y) of the half spectrum in place. */
static void xy_passes(const iho_fft3 *F, double *c, int sign)
{
    const int nx = F->nx, ny = F->ny, mz = F->nz / 2 + 1;
    const int nbz = (mz + PB - 1) / PB;
    const size_t maxn = (size_t)F->maxn;
    for (int pass = 0; pass < 2; ++pass) {
        /* forward: y then x ; backward: x then y (order is immaterial for the
           exact transform; this mirrors the separable row-column structure) */
        int axis_y = (sign < 0) ? (pass == 0) : (pass == 1);
        const int n = axis_y ? ny : nx;
        const int outer = axis_y ? nx : ny;
        const iho_cplan *P = axis_y ? &F->py : &F->px;
        const size_t stride = axis_y ? (size_t)mz : (size_t)ny * mz;
        #pragma omp parallel
        {
            double *buf = malloc(sizeof(double) * 2 * maxn * PB);
            double *work = malloc(sizeof(double) * 2 * maxn * PB);
            #pragma omp for collapse(2) schedule(static)
            for (int o = 0; o < outer; ++o) {
                for (int zb = 0; zb < nbz; ++zb) {
                    int z0 = zb * PB, b = mz - z0 < PB ? mz - z0 : PB;
                    size_t base = axis_y ? (size_t)o * ny * mz + z0 : (size_t)o * mz + z0;
                    for (int i = 0; i < n; ++i) {
                        const double *src = c + 2 * (base + (size_t)i * stride);
                        memcpy(buf + 2 * (size_t)i * b, src, sizeof(double) * 2 * b);
                    }
                    iho_cfft_batch(P, buf, work, b, sign);
                    for (int i = 0; i < n; ++i) {
                        double *dst = c + 2 * (base + (size_t)i * stride);
                        memcpy(dst, buf + 2 * (size_t)i * b, sizeof(double) * 2 * b);
                    }
                }
            }
            free(buf);
            free(work);
        }
    }
}

void iho_fft3_r2c(const iho_fft3 *F, const double *in, double *out)
{
    const int nx = F->nx, ny = F->ny, nz = F->nz, mz = nz / 2 + 1;
    const long rows = (long)nx * ny;
    const long nb = (rows + PB - 1) / PB;
    #pragma omp parallel
    {
        double *buf = malloc(sizeof(double) * 2 * (nz / 2 + 1) * PB);
        double *work = malloc(sizeof(double) * 2 * (nz / 2 + 1) * PB);
        #pragma omp for schedule(static)
        for (long bi = 0; bi < nb; ++bi) {
            long r0 = bi * PB;
            int b = rows - r0 < PB ? (int)(rows - r0) : PB;
            z_r2c_batch(F, in + (size_t)r0 * nz, out + 2 * (size_t)r0 * mz, b, buf, work);
        }
        free(buf);
        free(work);
    }
    xy_passes(F, out, -1);
}

void iho_fft3_c2r(const iho_fft3 *F, double *in_destroyed, double *out)
{
    const int nx = F->nx, ny = F->ny, nz = F->nz, mz = nz / 2 + 1;
    xy_passes(F, in_destroyed, +1);
    const long rows = (long)nx * ny;
    const long nb = (rows + PB - 1) / PB;
    #pragma omp parallel
    {
        double *buf = malloc(sizeof(double) * 2 * (nz / 2 + 1) * PB);
        double *work = malloc(sizeof(double) * 2 * (nz / 2 + 1) * PB);
        #pragma omp for schedule(static)
        for (long bi = 0; bi < nb; ++bi) {
            long r0 = bi * PB;
            int b = rows - r0 < PB ? (int)(rows - r0) : PB;
            z_c2r_batch(F, in_destroyed + 2 * (size_t)r0 * mz, out + (size_t)r0 * nz, b, buf, work);
        }
        free(buf);
        free(work);
    }
}
