// FFT plans and twiddle values shared by every spectral path of the library
// (the context path and the allocation-free correction), so that both use the
// same radix order and the same root table.
#pragma once

#include <math.h>
#include <string.h>

#include "evpg_common.cuh"

namespace evpg {

// Mixed-radix Stockham plan of length n: radices 8, 4, 2, 3, 5 in that order,
// then odd primes, each as often as it divides n.
inline void make_plan(int n, FftPlan& p) {
    memset(&p, 0, sizeof p);
    p.n = n;
    int m = n, nf = 0;
    const int pref[] = {8, 4, 2, 3, 5};
    for (int r : pref)
        while (m % r == 0 && nf < 12) {
            p.radix[nf++] = r;
            m /= r;
        }
    for (int q = 7; m > 1 && nf < 12; q += 2)
        while (m % q == 0 && nf < 12) {
            p.radix[nf++] = q;
            m /= q;
        }
    p.nf = nf;
    int ns = 1;
    for (int s = 0; s < nf; s++) {
        p.ns[s] = ns;
        ns *= p.radix[s];
    }
    plan_divisors(p);
}

// exp(-2 pi i t / n): the angle is reduced to the first octant in long double
// (exact values on the axes, quadrant symmetry), then rounded to double.
inline void unit_root(long t, long n, double* c, double* s) {
    t %= n;
    if (t < 0) t += n;
    const long q = (4 * t) / n, r = 4 * t - q * n;
    long double c0, s0;
    if (r == 0) {
        c0 = 1.0L;
        s0 = 0.0L;
    } else if (2 * r <= n) {
        const long double th = 1.57079632679489661923132169163975144L * ((long double)r / (long double)n);
        c0 = cosl(th);
        s0 = sinl(th);
    } else {
        const long double th = 1.57079632679489661923132169163975144L * ((long double)(n - r) / (long double)n);
        c0 = sinl(th);
        s0 = cosl(th);
    }
    long double cc, ss;
    switch (q & 3) {
        case 0: cc = c0; ss = s0; break;
        case 1: cc = -s0; ss = c0; break;
        case 2: cc = -c0; ss = -s0; break;
        default: cc = s0; ss = -c0; break;
    }
    *c = (double)cc;
    *s = -(double)ss;  // forward sign
}

}  // namespace evpg
