// Shared-memory Stockham FFT for batches of pencils (radix 8/4/2/3/5 and a
// generic O(p^2) stage for other primes). Replaces the FFTW 2 transforms of
// the reference (fftwnd_mpi, evolution.c:1163,1195): unnormalised, exponent
// sign -1 forward and +1 inverse.
//
// A CTA holds `npen` pencils of length n, pencil-major in shared memory, and
// runs all stages with two buffers (ping-pong), one __syncthreads per stage.
// Twiddles W_n^t = exp(-2 pi i t / n) come from a table in shared memory; the
// inverse uses their conjugates.
#pragma once
#include "evpg_common.cuh"

namespace evpg {

template <typename T, int SIGN>
__device__ __forceinline__ C2<T> mul_isign(C2<T> a) {
    // (SIGN*i) * a
    return SIGN < 0 ? mk<T>(a.y, -a.x) : mk<T>(-a.y, a.x);
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft4(C2<T>& a0, C2<T>& a1, C2<T>& a2, C2<T>& a3) {
    const C2<T> s02 = cadd<T>(a0, a2), d02 = csub<T>(a0, a2);
    const C2<T> s13 = cadd<T>(a1, a3), d13 = mul_isign<T, SIGN>(csub<T>(a1, a3));
    a0 = cadd<T>(s02, s13);
    a2 = csub<T>(s02, s13);
    a1 = cadd<T>(d02, d13);
    a3 = csub<T>(d02, d13);
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft8(C2<T>* v) {
    C2<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    C2<T> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<T, SIGN>(e0, e1, e2, e3);
    dft4<T, SIGN>(o0, o1, o2, o3);
    const T h = (T)0.70710678118654752440;
    // W8 = h(1 + SIGN i), W8^2 = SIGN i, W8^3 = h(-1 + SIGN i)
    const C2<T> w1 = mk<T>(h * (o1.x - (T)SIGN * o1.y), h * (o1.y + (T)SIGN * o1.x));
    const C2<T> w2 = mul_isign<T, SIGN>(o2);
    const C2<T> w3 = mk<T>(h * (-o3.x - (T)SIGN * o3.y), h * (-o3.y + (T)SIGN * o3.x));
    v[0] = cadd<T>(e0, o0); v[4] = csub<T>(e0, o0);
    v[1] = cadd<T>(e1, w1); v[5] = csub<T>(e1, w1);
    v[2] = cadd<T>(e2, w2); v[6] = csub<T>(e2, w2);
    v[3] = cadd<T>(e3, w3); v[7] = csub<T>(e3, w3);
}

// 16-point DFT as 4 x 4: inner DFT4 over q2 of v[q1 + 4 q2], twiddles
// W16^(q1 k2), outer DFT4 over q1; output V[4 k1 + k2] in natural order.
template <typename T, int SIGN>
__device__ __forceinline__ void dft16(C2<T>* v) {
    const T c1 = (T)0.92387953251128675613, s1 = (T)0.38268343236508977173;
    const T h = (T)0.70710678118654752440, sg = (T)SIGN;
#pragma unroll
    for (int q1 = 0; q1 < 4; q1++) dft4<T, SIGN>(v[q1], v[q1 + 4], v[q1 + 8], v[q1 + 12]);
    // v[q1 + 4 k2] now holds X[q1][k2]; multiply by W16^(q1 k2)
    const C2<T> w1 = mk<T>(c1, sg * s1), w2 = mk<T>(h, sg * h), w3 = mk<T>(s1, sg * c1);
    const C2<T> w6 = mk<T>(-h, sg * h), w9 = mk<T>(-c1, -sg * s1);
    v[5] = cmul<T>(v[5], w1);
    v[9] = cmul<T>(v[9], w2);
    v[13] = cmul<T>(v[13], w3);
    v[6] = cmul<T>(v[6], w2);
    v[10] = mul_isign<T, SIGN>(v[10]);
    v[14] = cmul<T>(v[14], w6);
    v[7] = cmul<T>(v[7], w3);
    v[11] = cmul<T>(v[11], w6);
    v[15] = cmul<T>(v[15], w9);
    C2<T> o[16];
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) {
        C2<T> a0 = v[4 * k2], a1 = v[4 * k2 + 1], a2 = v[4 * k2 + 2], a3 = v[4 * k2 + 3];
        dft4<T, SIGN>(a0, a1, a2, a3);
        o[k2] = a0;
        o[4 + k2] = a1;
        o[8 + k2] = a2;
        o[12 + k2] = a3;
    }
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = o[k];
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft3(C2<T>* v) {
    const T s = (T)SIGN * (T)0.86602540378443864676;
    const C2<T> t1 = cadd<T>(v[1], v[2]), t2 = csub<T>(v[1], v[2]);
    const C2<T> m = mk<T>(v[0].x - (T)0.5 * t1.x, v[0].y - (T)0.5 * t1.y);
    const C2<T> r = mk<T>(-s * t2.y, s * t2.x);  // i*s*t2
    v[0] = cadd<T>(v[0], t1);
    v[1] = cadd<T>(m, r);
    v[2] = csub<T>(m, r);
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft5(C2<T>* v) {
    const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
    const T s1 = (T)SIGN * (T)0.95105651629515357212, s2 = (T)SIGN * (T)0.58778525229247312917;
    const C2<T> a1 = cadd<T>(v[1], v[4]), b1 = csub<T>(v[1], v[4]);
    const C2<T> a2 = cadd<T>(v[2], v[3]), b2 = csub<T>(v[2], v[3]);
    const C2<T> x0 = v[0];
    const C2<T> m1 = mk<T>(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
    const C2<T> m2 = mk<T>(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
    const C2<T> q1 = mk<T>(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
    const C2<T> q2 = mk<T>(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
    // i*q = (-q.y, q.x)
    v[0] = mk<T>(x0.x + a1.x + a2.x, x0.y + a1.y + a2.y);
    v[1] = mk<T>(m1.x - q1.y, m1.y + q1.x);
    v[4] = mk<T>(m1.x + q1.y, m1.y - q1.x);
    v[2] = mk<T>(m2.x - q2.y, m2.y + q2.x);
    v[3] = mk<T>(m2.x + q2.y, m2.y - q2.x);
}

template <typename T, int SIGN>
__device__ __forceinline__ C2<T> twid(const C2<T>* tw, int t) {
    const C2<T> w = tw[t];
    return SIGN < 0 ? w : mk<T>(w.x, -w.y);
}

// Position of element p of a pencil in shared memory: with SKEW, p + p/16,
// which spreads the strided butterfly writes of the early Stockham stages
// over the banks (the pencil stride must then be at least n + n/16).
template <bool SKEW> __device__ __forceinline__ int fsk(int p) { return SKEW ? p + (p >> 4) : p; }
__host__ __device__ constexpr int skewed_len(int n) { return n + n / 16; }

// Run every stage of `pl` on npen pencils held in `a` (pencil p starts at
// element p*ps, ps >= n, or >= n + n/16 with SKEW; scratch `b` has the same
// layout). Returns the buffer holding the result. Must be called by all
// threads of the CTA; ends with a __syncthreads. R16: the plan may contain
// radix-16 stages (FP32 only; the 16-value buffer costs registers, so only the
// X pass, whose two-stage transforms of n = 128 gain most, is built with it).
template <typename T, int SIGN, bool SKEW = false, bool R16 = false>
__device__ C2<T>* fft_batch(C2<T>* a, C2<T>* b, int npen, int ps, const FftPlan& pl,
                            const C2<T>* tw) {
    const int n = pl.n;
    C2<T>* in = a;
    C2<T>* out = b;
    for (int s = 0; s < pl.nf; s++) {
        const int r = pl.radix[s], Ns = pl.ns[s], m = n / r, tws = n / (Ns * r);
        const int total = npen * m;
        const FastDiv dm = pl.dm[s], dns = pl.dns[s];
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int pen = dm.div(idx), j = idx - pen * m;
            const int jq = dns.div(j), jm = j - jq * Ns;
            const C2<T>* src = in + pen * ps;
            C2<T>* dst = out + pen * ps;
            const int d0 = jq * Ns * r + jm;
            constexpr bool W16 = R16 && sizeof(T) == 4;
            C2<T> v[W16 ? 16 : 8];
            if (W16 && r == 16) {
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    v[q] = src[fsk<SKEW>(j + q * m)];
                    if (q) v[q] = cmul<T>(v[q], twid<T, SIGN>(tw, q * jm * tws));
                }
                dft16<T, SIGN>(v);
#pragma unroll
                for (int q = 0; q < 16; q++) dst[fsk<SKEW>(d0 + q * Ns)] = v[q];
            } else if (r == 8) {
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    v[q] = src[fsk<SKEW>(j + q * m)];
                    if (q) v[q] = cmul<T>(v[q], twid<T, SIGN>(tw, q * jm * tws));
                }
                dft8<T, SIGN>(v);
#pragma unroll
                for (int q = 0; q < 8; q++) dst[fsk<SKEW>(d0 + q * Ns)] = v[q];
            } else if (r == 4) {
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    v[q] = src[fsk<SKEW>(j + q * m)];
                    if (q) v[q] = cmul<T>(v[q], twid<T, SIGN>(tw, q * jm * tws));
                }
                dft4<T, SIGN>(v[0], v[1], v[2], v[3]);
#pragma unroll
                for (int q = 0; q < 4; q++) dst[fsk<SKEW>(d0 + q * Ns)] = v[q];
            } else if (r == 2) {
                v[0] = src[fsk<SKEW>(j)];
                v[1] = cmul<T>(src[fsk<SKEW>(j + m)], twid<T, SIGN>(tw, jm * tws));
                dst[fsk<SKEW>(d0)] = cadd<T>(v[0], v[1]);
                dst[fsk<SKEW>(d0 + Ns)] = csub<T>(v[0], v[1]);
            } else if (r == 3) {
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    v[q] = src[fsk<SKEW>(j + q * m)];
                    if (q) v[q] = cmul<T>(v[q], twid<T, SIGN>(tw, q * jm * tws));
                }
                dft3<T, SIGN>(v);
#pragma unroll
                for (int q = 0; q < 3; q++) dst[fsk<SKEW>(d0 + q * Ns)] = v[q];
            } else if (r == 5) {
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    v[q] = src[fsk<SKEW>(j + q * m)];
                    if (q) v[q] = cmul<T>(v[q], twid<T, SIGN>(tw, q * jm * tws));
                }
                dft5<T, SIGN>(v);
#pragma unroll
                for (int q = 0; q < 5; q++) dst[fsk<SKEW>(d0 + q * Ns)] = v[q];
            } else {
                // generic prime radix: O(r^2) with the table (W_r^k = W_n^{k n/r})
                const int step = n / r;
                for (int q = 0; q < r; q++) {
                    C2<T> acc = mk<T>((T)0, (T)0);
                    for (int p = 0; p < r; p++) {
                        C2<T> x = src[fsk<SKEW>(j + p * m)];
                        if (p) x = cmul<T>(x, twid<T, SIGN>(tw, p * jm * tws));
                        acc = cadd<T>(acc, cmul<T>(x, twid<T, SIGN>(tw, ((p * q) % r) * step)));
                    }
                    dst[fsk<SKEW>(d0 + q * Ns)] = acc;
                }
            }
        }
        __syncthreads();
        C2<T>* t = in; in = out; out = t;
    }
    return in;
}

// Per-lane constants of the warp transforms, loaded once per kernel from the
// W_n^t table (they depend on the lane only): the twiddle of each cross-lane
// stage h = 16, 8, 4, 2 (1 on the low lane of a pair, whose result is not
// rotated), the sign +1 / -1 of the low / high lane of each stage
// h = 16 .. 1, and W_n^(l k2) for k2 = 1 .. EPL-1. The butterfly then reads
// p + s u (partner p, own value u: a + b on the low lane, a - b on the high
// lane) followed by one complex product, with no select between two results.
template <typename T, int EPL> struct WarpTw {
    C2<T> w[4];
    T s[5];
    C2<T> k[EPL > 1 ? EPL - 1 : 1];
    __device__ __forceinline__ void init(const C2<T>* tw, int lane) {
#pragma unroll
        for (int st = 0; st < 5; st++) {
            const int h = 16 >> st;
            const bool hi = (lane & h) != 0;
            s[st] = hi ? (T)-1 : (T)1;
            if (st < 4) w[st] = hi ? tw[(lane & (h - 1)) * (16 / h) * EPL] : mk<T>((T)1, (T)0);
        }
#pragma unroll
        for (int k2 = 1; k2 < EPL; k2++) k[k2 - 1] = tw[lane * k2];
    }
};

// a * w (SIGN < 0) or a * conj(w) (SIGN > 0)
template <typename T, int SIGN>
__device__ __forceinline__ C2<T> cmul_s(C2<T> a, C2<T> w) {
    return SIGN < 0 ? cmul<T>(a, w) : mk<T>(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}

// Warp-register FFT of length n = 32*EPL (EPL = 1, 2, 4 or 8): lane l holds
// x[l + 32 q] in v[q]. Four-step split n = EPL x 32: a length-EPL DFT in
// registers, twiddles W_n^(l k2), then for every k2 a 32-point radix-2
// decimation-in-frequency transform across the lanes with shuffles. On
// return lane l holds X[k2 + EPL * brev5(l)] in v[k2]. t: the lane's
// constants of the W_n^t table.
__device__ __forceinline__ int brev5(int l) { return (int)(__brev((unsigned)l) >> 27); }

template <typename T, int EPL, int SIGN>
__device__ __forceinline__ void warp_fft(C2<T> (&v)[EPL], const WarpTw<T, EPL>& t) {
    if (EPL == 2) {
        const C2<T> a = v[0], b = v[1];
        v[0] = cadd<T>(a, b);
        v[1] = csub<T>(a, b);
    } else if (EPL == 4) {
        dft4<T, SIGN>(v[0], v[1], v[2], v[3]);
    } else if (EPL == 8) {
        dft8<T, SIGN>(v);
    }
#pragma unroll
    for (int k2 = 1; k2 < EPL; k2++) v[k2] = cmul_s<T, SIGN>(v[k2], t.k[k2 - 1]);
#pragma unroll
    for (int st = 0; st < 5; st++) {
        const int h = 16 >> st;
#pragma unroll
        for (int k2 = 0; k2 < EPL; k2++) {
            const C2<T> u = v[k2];
            C2<T> r;
            r.x = __shfl_xor_sync(0xffffffffu, u.x, h);
            r.y = __shfl_xor_sync(0xffffffffu, u.y, h);
            r.x = fma(t.s[st], u.x, r.x);
            r.y = fma(t.s[st], u.y, r.y);
            v[k2] = st < 4 ? cmul_s<T, SIGN>(r, t.w[st < 4 ? st : 0]) : r;
        }
    }
}

// Inverse of warp_fft<T, EPL, -1>, unnormalised (n times the inverse): lane
// l holds X[k2 + EPL * brev5(l)] in v[k2] (the forward transform's output
// order); on return lane l holds x[l + 32 q] in v[q]. The forward steps
// undone in reverse: the cross-lane radix-2 stages from h = 1 up, each
// (A, B) = (a + b, (a - b) w) mapped back to (A + B conj(w), A - B conj(w)),
// then the conjugate twiddles and the length-EPL DFT with the opposite sign.
template <typename T, int EPL>
__device__ __forceinline__ void warp_ifft_brev(C2<T> (&v)[EPL], const WarpTw<T, EPL>& t) {
#pragma unroll
    for (int st = 4; st >= 0; st--) {
        const int h = 16 >> st;
#pragma unroll
        for (int k2 = 0; k2 < EPL; k2++) {
            const C2<T> u = st < 4 ? cmul_s<T, 1>(v[k2], t.w[st < 4 ? st : 0]) : v[k2];
            C2<T> p;
            p.x = __shfl_xor_sync(0xffffffffu, u.x, h);
            p.y = __shfl_xor_sync(0xffffffffu, u.y, h);
            v[k2] = mk<T>(fma(t.s[st], u.x, p.x), fma(t.s[st], u.y, p.y));
        }
    }
#pragma unroll
    for (int k2 = 1; k2 < EPL; k2++) v[k2] = cmul_s<T, 1>(v[k2], t.k[k2 - 1]);
    if (EPL == 2) {
        const C2<T> a = v[0], b = v[1];
        v[0] = cadd<T>(a, b);
        v[1] = csub<T>(a, b);
    } else if (EPL == 4) {
        dft4<T, 1>(v[0], v[1], v[2], v[3]);
    } else if (EPL == 8) {
        dft8<T, 1>(v);
    }
}

}  // namespace evpg
