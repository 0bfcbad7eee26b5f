/*
 * CPU mixed-radix complex DFT (oracle test infrastructure; see fft_cpu.h).
 * Plain C, no architecture intrinsics; built with -ffp-contract=off so x86
 * and Arm hosts give identical bits.
 */
#include "fft_cpu.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define SRX_MAX_FACTORS 64

/* cos/sin of 2*pi*k/n with exact values on the axes and quadrant symmetry. */
static void unit_root(long k, long n, double *c, double *s)
{
    long q, r;
    double c0, s0, th;
    k %= n;
    if (k < 0) k += n;
    q = (4 * k) / n;
    r = 4 * k - q * n; /* angle = (q + r/n) * pi/2, 0 <= r < n */
    if (r == 0) {
        c0 = 1.0;
        s0 = 0.0;
    } else if (2 * r <= n) {
        th = M_PI_2 * ((double)r / (double)n);
        c0 = cos(th);
        s0 = sin(th);
    } else {
        th = M_PI_2 * ((double)(n - r) / (double)n);
        c0 = sin(th);
        s0 = cos(th);
    }
    switch (q & 3) {
    case 0: *c = c0;  *s = s0;  break;
    case 1: *c = -s0; *s = c0;  break;
    case 2: *c = -c0; *s = -s0; break;
    default: *c = s0; *s = -c0; break;
    }
}

static int factorize(int n, int *f)
{
    int nf = 0, p;
    while (n % 4 == 0) { f[nf++] = 4; n /= 4; }
    while (n % 2 == 0) { f[nf++] = 2; n /= 2; }
    for (p = 3; n > 1; p += 2) {
        while (n % p == 0) {
            if (nf >= SRX_MAX_FACTORS) return -1;
            f[nf++] = p;
            n /= p;
        }
    }
    return nf;
}

typedef struct {
    int n, nf, sign;
    int f[SRX_MAX_FACTORS];
    double *w; /* 2*n: w[k] = exp(sign*2*pi*i*k/n) */
} plan1d;

static int plan_make(plan1d *p, int n, int sign)
{
    long k;
    p->n = n;
    p->sign = sign;
    p->nf = factorize(n, p->f);
    if (p->nf < 0) return -1;
    p->w = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    if (!p->w) return -1;
    for (k = 0; k < n; k++) {
        double c, s;
        unit_root(k, n, &c, &s);
        p->w[2 * k] = c;
        p->w[2 * k + 1] = sign < 0 ? -s : s;
    }
    return 0;
}

/* One Stockham stage of radix r with Ns = product of the earlier radices. */
static void stage(const plan1d *p, const double *in, double *out, int r, int Ns)
{
    const int n = p->n, np = n / r, tws = n / (Ns * r), rs = n / r;
    double v[2 * 64], V[2 * 64];
    int j, a, b;
    for (j = 0; j < np; j++) {
        const int jm = j % Ns;
        const int idxD = (j / Ns) * Ns * r + jm;
        for (a = 0; a < r; a++) {
            const double xr = in[2 * (j + a * np)], xi = in[2 * (j + a * np) + 1];
            const long t = ((long)a * jm * tws) % n;
            const double wr = p->w[2 * t], wi = p->w[2 * t + 1];
            v[2 * a] = xr * wr - xi * wi;
            v[2 * a + 1] = xr * wi + xi * wr;
        }
        if (r == 2) {
            V[0] = v[0] + v[2]; V[1] = v[1] + v[3];
            V[2] = v[0] - v[2]; V[3] = v[1] - v[3];
        } else if (r == 4) {
            /* exp(sign*2*pi*i/4) = sign*i */
            const double s = (double)p->sign;
            const double ar = v[0] + v[4], ai = v[1] + v[5];
            const double br = v[0] - v[4], bi = v[1] - v[5];
            const double cr = v[2] + v[6], ci = v[3] + v[7];
            const double dr = v[2] - v[6], di = v[3] - v[7];
            V[0] = ar + cr;      V[1] = ai + ci;
            V[4] = ar - cr;      V[5] = ai - ci;
            /* (sign*i) * d = (-sign*di, sign*dr) */
            V[2] = br - s * di;  V[3] = bi + s * dr;
            V[6] = br + s * di;  V[7] = bi - s * dr;
        } else {
            for (b = 0; b < r; b++) {
                double sr = 0.0, si = 0.0;
                for (a = 0; a < r; a++) {
                    const long t = (long)((a * b) % r) * rs;
                    const double wr = p->w[2 * t], wi = p->w[2 * t + 1];
                    sr += v[2 * a] * wr - v[2 * a + 1] * wi;
                    si += v[2 * a] * wi + v[2 * a + 1] * wr;
                }
                V[2 * b] = sr;
                V[2 * b + 1] = si;
            }
        }
        for (b = 0; b < r; b++) {
            out[2 * (idxD + b * Ns)] = V[2 * b];
            out[2 * (idxD + b * Ns) + 1] = V[2 * b + 1];
        }
    }
}

int srx_fft1d_many(double *data, int n, int howmany, long stride, long dist, int sign)
{
    plan1d p;
    double *x, *y;
    int h, i, s, Ns;
    if (n < 1 || howmany < 0 || (sign != 1 && sign != -1)) return -1;
    if (n == 1 || howmany == 0) return 0;
    if (plan_make(&p, n, sign)) return -1;
    for (s = 0; s < p.nf; s++)
        if (p.f[s] > 64) { free(p.w); return -1; }
    x = (double *)malloc(sizeof(double) * 4 * (size_t)n);
    if (!x) { free(p.w); return -1; }
    y = x + 2 * n;
    for (h = 0; h < howmany; h++) {
        double *base = data + 2 * (size_t)h * (size_t)dist;
        double *src = x, *dst = y, *tmp;
        for (i = 0; i < n; i++) {
            src[2 * i] = base[2 * (size_t)i * (size_t)stride];
            src[2 * i + 1] = base[2 * (size_t)i * (size_t)stride + 1];
        }
        Ns = 1;
        for (s = 0; s < p.nf; s++) {
            stage(&p, src, dst, p.f[s], Ns);
            Ns *= p.f[s];
            tmp = src; src = dst; dst = tmp;
        }
        for (i = 0; i < n; i++) {
            base[2 * (size_t)i * (size_t)stride] = src[2 * i];
            base[2 * (size_t)i * (size_t)stride + 1] = src[2 * i + 1];
        }
    }
    free(x);
    free(p.w);
    return 0;
}

int srx_fft3d(double *data, int n0, int n1, int n2, int sign)
{
    int x;
    const long n12 = (long)n1 * n2;
    if (srx_fft1d_many(data, n2, n0 * n1, 1, n2, sign)) return -1;
    for (x = 0; x < n0; x++)
        if (srx_fft1d_many(data + 2 * (size_t)x * (size_t)n12, n1, n2, n2, 1, sign)) return -1;
    if (srx_fft1d_many(data, n0, (int)n12, n12, 1, sign)) return -1;
    return 0;
}
