/*
 * gsl/gsl_rng.h (shim) -- GSL's random-number interface as the reference's
 * src/setup.c uses it (setup.c:77, 117-126, 1179-1184, 1283): the MT19937
 * generator of Matsumoto and Nishimura, seeded and read the way GSL documents
 * it (gsl_rng_set with the 2002 initialisation, seed 0 meaning 4357;
 * gsl_rng_uniform = next 32-bit output / 2^32).  TEST INFRASTRUCTURE ONLY
 * (the second oracle, oracle/_ref); GSL (the reference names version 2.1,
 * src/Makefile:7-8) is not installed here.
 */
#ifndef IH_REF_SHIM_GSL_RNG_H
#define IH_REF_SHIM_GSL_RNG_H

typedef struct {
    const char *name;
    unsigned long max, min;
} gsl_rng_type;

typedef struct gsl_rng gsl_rng;

extern const gsl_rng_type *gsl_rng_mt19937;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long seed);
void gsl_rng_free(gsl_rng *r);
unsigned long gsl_rng_get(const gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);

#endif
