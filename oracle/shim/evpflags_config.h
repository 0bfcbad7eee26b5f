/*
 * Compile-time configuration for the oracle build of the reference.
 *
 * TEST INFRASTRUCTURE ONLY. Pre-included (gcc -include) before every
 * reference translation unit. It defines EVPFLAGS_H, so the reference's own
 * evpFlags.h (evpFlags.h:1-46) is skipped by its include guard, and it sets
 * the same macros with one change: DD_CU is left undefined, so the elastic
 * constants come from the namelist's ElastConst_PhaseI instead of the
 * temperature formula at init.c:822-826 (the reference README.txt:2 allows
 * this). Every other flag matches evpFlags.h as shipped; the optional
 * flavours switch on NR_MODIFIED (SRX_ORACLE_NR_MODIFIED), DD_POWER_LAW
 * (SRX_ORACLE_POWER_LAW) and DD_GND with its DD_GND_FIRST_ORDER companion
 * (SRX_ORACLE_GND), all commented-out options of evpFlags.h.
 */
#ifndef EVPFLAGS_H
#define EVPFLAGS_H

#define NPHMAX 2
#define NSYSMX 12

#define DD_BASED_FLAG
#ifdef DD_BASED_FLAG
/* DD_CU intentionally off (see header comment). */
#define FORWARD_PLUS_BACKWARD
#ifdef SRX_ORACLE_NR_MODIFIED
#define NR_MODIFIED /* line-search NR of the FFTW3 variant */
#endif
#ifdef SRX_ORACLE_POWER_LAW
#define DD_POWER_LAW /* power-law flow rule instead of the sinh law (evpFlags.h:24) */
#endif
#ifdef SRX_ORACLE_GND
#define DD_GND /* geometrically necessary dislocations (evpFlags.h:29-32) */
#define DD_GND_FIRST_ORDER
#endif
#define PF_DRX
#ifdef PF_DRX
#define GB_BULGING_ONLY
#endif
#endif

#endif
