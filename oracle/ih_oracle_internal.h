/* ih_oracle_internal.h -- private declarations of the CPU oracle (test
 * infrastructure only; see ih_oracle.h). */
#ifndef IH_ORACLE_INTERNAL_H
#define IH_ORACLE_INTERNAL_H

#include <stddef.h>
#include "ih_oracle.h"

typedef struct {
    int n, nst;
    int radix[40];
    double *tw[40];
} iho_cplan;

typedef struct {
    int nx, ny, nz, maxn;
    iho_cplan px, py, pz; /* pz has length nz/2 */
    double *wz;           /* exp(-2 pi i k/nz), k = 0..nz/2 */
} iho_fft3;

int iho_cplan_init(iho_cplan *p, int n);
void iho_cplan_free(iho_cplan *p);
void iho_cfft_batch(const iho_cplan *p, double *x, double *work, int b, int sign);
int iho_fft3_init(iho_fft3 *F, int nx, int ny, int nz);
void iho_fft3_free(iho_fft3 *F);
void iho_fft3_r2c(const iho_fft3 *F, const double *in, double *out);
void iho_fft3_c2r(const iho_fft3 *F, double *in_destroyed, double *out);

#endif
