/*
 * Stand-in for the GSL random-number interface that SRX declares.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/_ref build). In the reference the generator
 * only feeds kappa_drx (init.c:1011-1014,1052-1057), which the compiled-in
 * code never reads, so a small deterministic generator is enough.
 */
#ifndef SRX_SHIM_GSL_RNG_H
#define SRX_SHIM_GSL_RNG_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct { const char *name; } gsl_rng_type;
typedef struct { unsigned long long state; } gsl_rng;

extern const gsl_rng_type *gsl_rng_default;
extern unsigned long gsl_rng_default_seed;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_free(gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);

#ifdef __cplusplus
}
#endif
#endif
