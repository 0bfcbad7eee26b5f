/*
 * Stand-in for the one GSL distribution SRX calls (init.c:1054).
 * TEST INFRASTRUCTURE ONLY (oracle/_ref build); the value is never read.
 */
#ifndef SRX_SHIM_GSL_RANDIST_H
#define SRX_SHIM_GSL_RANDIST_H
#include <gsl/gsl_rng.h>
#ifdef __cplusplus
extern "C" {
#endif

double gsl_ran_weibull(const gsl_rng *r, double a, double b);

#ifdef __cplusplus
}
#endif
#endif
