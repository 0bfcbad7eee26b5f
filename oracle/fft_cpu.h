/*
 * CPU mixed-radix complex DFT (oracle test infrastructure).
 *
 * Stands in for FFTW 2.1.5 (Makefile:9-11 of the reference; not vendored,
 * version pinned only by that path) at the reference's call sites
 * evolution.c:1163,1195. Restates the published definition
 *   X[k] = sum_j x[j] exp(sign * 2*pi*i * j*k / n)
 * unnormalised, evaluated by a Stockham autosort with radix 4/2/3/5 stages and
 * an O(p^2) stage for any other prime factor p. Pinned against numpy.fft.fftn.
 */
#ifndef SRX_ORACLE_FFT_CPU_H
#define SRX_ORACLE_FFT_CPU_H
#ifdef __cplusplus
extern "C" {
#endif

/* In-place 3-D transform of interleaved complex data laid out [n0][n1][n2]
 * (n2 fastest). sign = -1 forward, +1 backward. Returns 0 on success. */
int srx_fft3d(double *data, int n0, int n1, int n2, int sign);

/* In-place 1-D transform of `howmany` interleaved complex sequences of length
 * n, element stride `stride` (in complex elements), sequence distance `dist`. */
int srx_fft1d_many(double *data, int n, int howmany, long stride, long dist, int sign);

#ifdef __cplusplus
}
#endif
#endif
