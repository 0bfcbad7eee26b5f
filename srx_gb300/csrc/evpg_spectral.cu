// Spectral-chain kernels (see evpg_spectral.cuh) and their launcher.
#include "evpg_ctx.h"
#include "evpg_spectral.cuh"
#include "evpg_plan.h"

#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

namespace evpg {

template <typename T>
__device__ __forceinline__ void load_tw(C2<T>* tw, const C2<T>* src, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) tw[i] = src[i];
}

// Asynchronous global -> shared copy of one complex element (cp.async, 8 or
// 16 bytes, both addresses aligned to the element size); completes at
// cp_async_wait_all.
template <typename T>
__device__ __forceinline__ void cp_async_elem(C2<T>* dst, const C2<T>* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(src), "n"(sizeof(C2<T>))
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Shared-memory layout of the Stockham passes: FP32 pencils are skewed (fsk),
// which removes the bank conflicts of the early stages; FP64 pencils, whose
// passes are bound by the FP64 pipe, keep the plain layout and its smaller
// footprint. Pencil strides for element size es of a complex value: x and y
// passes (odd), z passes.
__host__ __device__ constexpr bool x_skew(size_t es) { return es == 8; }
__host__ __device__ constexpr int x_pencil_stride(int n, size_t es) { return x_skew(es) ? skewed_len(n) | 1 : n + 1; }
__host__ __device__ constexpr int z_pencil_stride(int n, size_t es) { return x_skew(es) ? skewed_len(n) | 1 : n; }

// Forward z: three complex FFTs of (sig[2p] + i sig[2p+1]) per column, split
// into the two half spectra. bid: CTA index within this RVE's grid.
template <typename T>
__device__ __forceinline__ void fwd_z_body(const ZArgs<T>& a, int bid, unsigned char* smem) {
    const Grid& g = a.g;
    constexpr bool SK = x_skew(sizeof(C2<T>));
    const int n = g.n2, nh = g.nh, P = a.P, ps = z_pencil_stride(n, sizeof(C2<T>));
    C2<T>* tw = reinterpret_cast<C2<T>*>(smem);
    C2<T>* bA = tw + n;
    C2<T>* bB = bA + P * ps;
    const int ncol = g.n0 * g.n1, c0 = bid * P, np = min(P, ncol - c0);
    load_tw<T>(tw, a.tw, n);
    for (int pair = 0; pair < 3; pair++) {
        const T* sa = a.sig + (size_t)(2 * pair) * g.N + (size_t)c0 * n;
        const T* sb = a.sig + (size_t)(2 * pair + 1) * g.N + (size_t)c0 * n;
        for (int i = threadIdx.x; i < np * n; i += blockDim.x) {
            const int col = a.dn.div(i), k = i - col * n;
            bA[col * ps + fsk<SK>(k)] = mk<T>(sa[i], sb[i]);
        }
        __syncthreads();
        const C2<T>* r = fft_batch<T, -1, SK>(bA, bB, np, ps, a.pl, tw);
        C2<T>* oa = a.spec + (size_t)(2 * pair) * g.Nh + (size_t)c0 * nh;
        C2<T>* ob = a.spec + (size_t)(2 * pair + 1) * g.Nh + (size_t)c0 * nh;
        for (int i = threadIdx.x; i < np * nh; i += blockDim.x) {
            const int col = a.dnh.div(i), k = i - col * nh;
            const C2<T> z = r[col * ps + fsk<SK>(k)];
            const C2<T> w = r[col * ps + fsk<SK>(k == 0 ? 0 : n - k)];
            // A = (Z(k) + conj Z(n-k))/2, B = (Z(k) - conj Z(n-k))/(2i)
            oa[i] = mk<T>((T)0.5 * (z.x + w.x), (T)0.5 * (z.y - w.y));
            ob[i] = mk<T>((T)0.5 * (z.y + w.y), (T)-0.5 * (z.x - w.x));
        }
        __syncthreads();
    }
}

// c2c along y on ncomp planes, pencils (x, kz..kz+P).
template <typename T, int SIGN>
__device__ __forceinline__ void y_body(const YArgs<T>& a, int bid, unsigned char* smem) {
    const Grid& g = a.g;
    constexpr bool SK = x_skew(sizeof(C2<T>));
    const int n = g.n1, ps = x_pencil_stride(n, sizeof(C2<T>)), P = a.P, nh = g.nh;
    C2<T>* tw = reinterpret_cast<C2<T>*>(smem);
    C2<T>* bA = tw + n;
    C2<T>* bB = bA + P * ps;
    const int ntile = (nh + P - 1) / P;
    const int x = bid / ntile, kz0 = (bid % ntile) * P, np = min(P, nh - kz0);
    const FastDiv dq = a.dnp[np == P ? 0 : 1];
    load_tw<T>(tw, a.tw, n);
    for (int c = 0; c < a.ncomp; c++) {
        C2<T>* base = a.spec + (size_t)c * g.Nh + (size_t)x * n * nh + kz0;
        for (int i = threadIdx.x; i < n * np; i += blockDim.x) {
            const int y = dq.div(i), kk = i - y * np;
            cp_async_elem<T>(bA + kk * ps + fsk<SK>(y), base + (size_t)y * nh + kk);
        }
        cp_async_wait_all();
        __syncthreads();
        const C2<T>* r = fft_batch<T, SIGN, SK>(bA, bB, np, ps, a.pl, tw);
        for (int i = threadIdx.x; i < n * np; i += blockDim.x) {
            const int y = dq.div(i), kk = i - y * np;
            base[(size_t)y * nh + kk] = r[kk * ps + fsk<SK>(y)];
        }
        __syncthreads();
    }
}

// Forward x, Green contraction, inverse x on pencils (y, kz..kz+P).
// Green correction du(k) = Gamma(k) : sig_hat(k) at one wave vector, with the
// k = 0 term, and on the Nyquist planes the Hermitian part
// (du(k) + conj du(-k))/2 with sig_hat(-k) = conj sig_hat(k).
template <typename T, bool SHARED_C0>
__device__ __forceinline__ void green_point(const GreenK<T>& gk, const Grid& g, const T (&rn)[3], int kx,
                                            int ky, int kz, const C2<T> (&sb)[6], C2<T> (&du)[9]) {
    if ((kx | ky | kz) == 0) {
        green_k0<T>(gk.s0, gk.elast_bc, sb, du);
        return;
    }
    T nv[3];
    kvec<T>(kx, ky, kz, g, rn, nv);
    if (SHARED_C0) green_du<T>(C0Shared<T>{&gk.c0[0][0][0][0]}, nv, sb, du);
    else green_du<T>(C0Param<T>{gk.c0}, nv, sb, du);
    const bool nyq = ((g.n0 & 1) == 0 && 2 * kx == g.n0) ||
                     ((g.n1 & 1) == 0 && 2 * ky == g.n1) ||
                     ((g.n2 & 1) == 0 && 2 * kz == g.n2);
    if (nyq) {
        C2<T> sm[6], dm[9];
#pragma unroll
        for (int c = 0; c < 6; c++) sm[c] = cconj<T>(sb[c]);
        const int mx = (g.n0 - kx) % g.n0, my = (g.n1 - ky) % g.n1, mz = (g.n2 - kz) % g.n2;
        kvec<T>(mx, my, mz, g, rn, nv);
        if (SHARED_C0) green_du<T>(C0Shared<T>{&gk.c0[0][0][0][0]}, nv, sm, dm);
        else green_du<T>(C0Param<T>{gk.c0}, nv, sm, dm);
#pragma unroll
        for (int c = 0; c < 9; c++)
            du[c] = mk<T>((T)0.5 * (du[c].x + dm[c].x), (T)0.5 * (du[c].y - dm[c].y));
    }
}

template <typename T, bool SHARED_C0>
__device__ __forceinline__ void x_green_body(const XArgs<T>& a, const GreenK<T>& gk, int bid,
                                             unsigned char* smem) {
    const Grid& g = a.g;
    constexpr bool SK = x_skew(sizeof(C2<T>));
    const int n = g.n0, ps = x_pencil_stride(n, sizeof(C2<T>)), P = a.P, nh = g.nh;
    C2<T>* tw = reinterpret_cast<C2<T>*>(smem);
    C2<T>* bA = tw + n;
    C2<T>* bB = bA + 9 * P * ps;
    const int ntile = (nh + P - 1) / P;
    const int y = bid / ntile, kz0 = (bid % ntile) * P, np = min(P, nh - kz0);
    const size_t xs = (size_t)g.n1 * nh;
    const T rn[3] = {gk.rn[0], gk.rn[1], gk.rn[2]};
    const int tile = np == P ? 0 : 1;
    const FastDiv dq = a.dnp[tile], dnq = a.dnnp[tile];
    load_tw<T>(tw, a.tw, n);
    for (int i = threadIdx.x; i < 6 * n * np; i += blockDim.x) {
        const int c = dnq.div(i), rem = i - c * n * np, x = dq.div(rem), kk = rem - x * np;
        cp_async_elem<T>(bA + (c * np + kk) * ps + fsk<SK>(x), a.spec + (size_t)c * g.Nh + x * xs + (size_t)y * nh + kz0 + kk);
    }
    cp_async_wait_all();
    __syncthreads();
    C2<T>* R = fft_batch<T, -1, SK, true>(bA, bB, 6 * np, ps, a.pl, tw);
    C2<T>* W = (R == bA) ? bB : bA;
    for (int i = threadIdx.x; i < n * np; i += blockDim.x) {
        const int kk = a.dn.div(i), kx = i - kk * n, kz = kz0 + kk, ky = y;
        C2<T> sb[6], du[9];
#pragma unroll
        for (int c = 0; c < 6; c++) sb[c] = R[(c * np + kk) * ps + fsk<SK>(kx)];
        green_point<T, SHARED_C0>(gk, g, rn, kx, ky, kz, sb, du);
#pragma unroll
        for (int c = 0; c < 9; c++) W[(c * np + kk) * ps + fsk<SK>(kx)] = du[c];
    }
    __syncthreads();
    const C2<T>* R2 = fft_batch<T, 1, SK, true>(W, (W == bA) ? bB : bA, 9 * np, ps, a.pl, tw);
    for (int i = threadIdx.x; i < 9 * n * np; i += blockDim.x) {
        const int c = dnq.div(i), rem = i - c * n * np, x = dq.div(rem), kk = rem - x * np;
        a.spec[(size_t)c * g.Nh + x * xs + (size_t)y * nh + kz0 + kk] = R2[(c * np + kk) * ps + fsk<SK>(x)];
    }
}

// X pass as warp-register transforms (FP32, n0 = 32 E with E in {1, 2, 4}).
// A CTA takes XW_PEN consecutive pencils of the flattened (y, kz) index (one
// x-row of the spectrum holds them contiguously), one warp per pencil with
// the six stress components in registers (lane l holds x = l + 32 q): the
// forward transforms, the Green contraction at the lane's E wave numbers and
// the nine inverse transforms use shared memory only for the coalesced
// global loads and stores. The [component][x][pencil] tile has padded rows
// (8-byte column reads without bank conflicts), and every warp reads and
// writes its own column, so no barrier separates the forward and inverse work.
constexpr int XW_PEN = 8;
constexpr int XW_ROW = XW_PEN + 1;
constexpr int XW_THREADS = 32 * XW_PEN;

__host__ __device__ constexpr bool xw_eligible(int n0, size_t es) {
    return es == 8 && (n0 == 32 || n0 == 64 || n0 == 128);
}
// rows: components the tile holds (9; 6 when the antisymmetric part is deferred)
__host__ __device__ constexpr size_t xw_smem(int n0, size_t es, int rows = 9) {
    return (size_t)(n0 + rows * n0 * XW_ROW) * es;
}

template <typename T, int E, bool SHARED_C0>
__device__ __forceinline__ void x_warp_body(const XArgs<T>& a, const GreenK<T>& gk, int bid, unsigned char* smem) {
    const Grid& g = a.g;
    constexpr int n = 32 * E, LOGN = E == 1 ? 5 : E == 2 ? 6 : 7;
    const int nh = g.nh;
    C2<T>* tw = reinterpret_cast<C2<T>*>(smem);
    C2<T>* tile = tw + n;
    const int p0 = bid * XW_PEN, np = min(XW_PEN, g.n1 * nh - p0);
    const size_t xs = (size_t)g.n1 * nh;
    const T rn[3] = {gk.rn[0], gk.rn[1], gk.rn[2]};
    const int mode = a.mode;
    // tile rows inverse-transformed along x and stored: [clo, chi), stored as
    // spectrum components coff + row (the flush keeps the three deferred
    // components in rows 0..2, so the deferring form's tile holds six rows)
    const int clo = 0, chi = mode == XM_DEFER ? 6 : mode == XM_FLUSH ? 3 : 9, coff = mode == XM_FLUSH ? 6 : 0;
    load_tw<T>(tw, a.tw, n);
    if (mode != XM_FLUSH)
        for (int i = threadIdx.x; i < 6 * n * XW_PEN; i += blockDim.x) {
            const int kk = i % XW_PEN, row = i / XW_PEN, c = row >> LOGN, x = row & (n - 1);
            if (kk < np) cp_async_elem<T>(tile + row * XW_ROW + kk, a.spec + (size_t)c * g.Nh + x * xs + p0 + kk);
        }
    cp_async_wait_all();
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (w < np) {
        const int p = p0 + w, ky = a.dnh.div(p), kz = p - ky * nh;
        C2<T>* col = tile + w;
        WarpTw<T, E> wt;
        wt.init(tw, lane);
        // the deferred components of this pencil, in the lane order of du:
        // written to the pending buffer (XM_DEFER), read from the sum (XM_FLUSH)
        const size_t npen = (size_t)g.n1 * nh;
        C2<T>* dbuf = a.dbuf ? a.dbuf + (size_t)p * n + lane : nullptr;
        if (mode != XM_FLUSH) {
            // one component at a time in registers: forward transform, back to
            // its column in the transform's output order
#pragma unroll 1
            for (int c = 0; c < 6; c++) {
                C2<T> v[E];
#pragma unroll
                for (int q = 0; q < E; q++) v[q] = col[(c * n + lane + 32 * q) * XW_ROW];
                warp_fft<T, E, -1>(v, wt);
#pragma unroll
                for (int q = 0; q < E; q++) col[(c * n + lane + 32 * q) * XW_ROW] = v[q];
            }
            // lane l holds kx = k2 + E brev5(l) in slot k2; du goes to the same
            // slots, which the inverse transforms read back in that order
            const int kb = E * brev5(lane);
#pragma unroll 1
            for (int k2 = 0; k2 < E; k2++) {
                C2<T> sb[6], du[9];
#pragma unroll
                for (int c = 0; c < 6; c++) sb[c] = col[(c * n + lane + 32 * k2) * XW_ROW];
                green_point<T, SHARED_C0>(gk, g, rn, k2 + kb, ky, kz, sb, du);
                if (mode == XM_DEFER) {
#pragma unroll
                    for (int c = 0; c < 6; c++) col[(c * n + lane + 32 * k2) * XW_ROW] = du[c];
#pragma unroll
                    for (int c = 6; c < 9; c++) dbuf[(size_t)(c - 6) * npen * n + 32 * k2] = du[c];
                } else {
#pragma unroll
                    for (int c = 0; c < 9; c++) col[(c * n + lane + 32 * k2) * XW_ROW] = du[c];
                }
            }
        } else {
#pragma unroll
            for (int c = 0; c < 3; c++)
#pragma unroll
                for (int q = 0; q < E; q++)
                    col[(c * n + lane + 32 * q) * XW_ROW] = dbuf[(size_t)c * npen * n + 32 * q];
        }
#pragma unroll 1
        for (int c = clo; c < chi; c++) {
            C2<T> u[E];
#pragma unroll
            for (int q = 0; q < E; q++) u[q] = col[(c * n + lane + 32 * q) * XW_ROW];
            warp_ifft_brev<T, E>(u, wt);
#pragma unroll
            for (int q = 0; q < E; q++) col[(c * n + lane + 32 * q) * XW_ROW] = u[q];
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < (chi - clo) * n * XW_PEN; i += blockDim.x) {
        const int kk = i % XW_PEN, row = clo * n + i / XW_PEN, c = coff + (row >> LOGN), x = row & (n - 1);
        if (kk < np) a.spec[(size_t)c * g.Nh + x * xs + p0 + kk] = tile[row * XW_ROW + kk];
    }
}

// Inverse z: pairs of Hermitian half spectra -> one complex IFFT -> two real
// fields; DisGrad += dE + re/N (evolution.c:1197). The DisGrad values of a
// pair are loaded into registers before its transform, so their latency
// overlaps the FFT stages (at most INVZ_EPT elements per thread).
constexpr int INVZ_EPT = 16;

template <typename T>
__device__ __forceinline__ void inv_z_body(const ZArgs<T>& a, int bid, unsigned char* smem) {
    const Grid& g = a.g;
    constexpr bool SK = x_skew(sizeof(C2<T>));
    const int n = g.n2, nh = g.nh, P = a.P, ps = z_pencil_stride(n, sizeof(C2<T>));
    C2<T>* tw = reinterpret_cast<C2<T>*>(smem);
    C2<T>* bA = tw + n;
    C2<T>* bB = bA + P * ps;
    const int ncol = g.n0 * g.n1, c0 = bid * P, np = min(P, ncol - c0);
    const int tot = np * n;
    load_tw<T>(tw, a.tw, n);
    for (int pair = 0; pair < 5; pair++) {
        const int ca = 2 * pair, cb = 2 * pair + 1;
        const bool hasb = cb < 9;
        T* da = a.dg + (size_t)ca * g.N + (size_t)c0 * n;
        T* db = a.dg + (size_t)(hasb ? cb : ca) * g.N + (size_t)c0 * n;
        T pa[INVZ_EPT], pb[INVZ_EPT];
#pragma unroll
        for (int e = 0; e < INVZ_EPT; e++) {
            const int i = threadIdx.x + e * blockDim.x;
            pa[e] = (i < tot) ? da[i] : (T)0;
            pb[e] = (i < tot && hasb) ? db[i] : (T)0;
        }
        const C2<T>* sa = a.spec + (size_t)ca * g.Nh + (size_t)c0 * nh;
        const C2<T>* sb = a.spec + (size_t)(hasb ? cb : ca) * g.Nh + (size_t)c0 * nh;
        for (int i = threadIdx.x; i < tot; i += blockDim.x) {
            const int col = a.dn.div(i), k = i - col * n;
            C2<T> z;
            if (k < nh) {
                const C2<T> u = sa[col * nh + k];
                const C2<T> v = hasb ? sb[col * nh + k] : mk<T>((T)0, (T)0);
                z = mk<T>(u.x - v.y, u.y + v.x);  // u + i v
            } else {
                const C2<T> u = sa[col * nh + (n - k)];
                const C2<T> v = hasb ? sb[col * nh + (n - k)] : mk<T>((T)0, (T)0);
                z = mk<T>(u.x + v.y, -u.y + v.x);  // conj u + i conj v
            }
            bA[col * ps + fsk<SK>(k)] = z;
        }
        __syncthreads();
        const C2<T>* r = fft_batch<T, 1, SK>(bA, bB, np, ps, a.pl, tw);
        const T ea = (T)a.dE9[ca], eb = hasb ? (T)a.dE9[cb] : (T)0;
#pragma unroll
        for (int e = 0; e < INVZ_EPT; e++) {
            const int i = threadIdx.x + e * blockDim.x;
            if (i < tot) {
                const int col = a.dn.div(i), k = i - col * n;
                const C2<T> z = r[col * ps + fsk<SK>(k)];
                da[i] = pa[e] + (ea + z.x * a.invN);
                if (hasb) db[i] = pb[e] + (eb + z.y * a.invN);
            }
        }
        __syncthreads();
    }
}

// ---- fused z+y passes on x planes (power-of-two n1 == n2 = 32*E)
//
// One CTA per (x plane, component). Forward: every warp takes pairs of z rows
// (2j, 2j+1) of the component, loads row 2j + i row 2j+1 (coalesced),
// transforms it in registers and splits the two rows' half spectra through a
// per-warp row buffer into the shared half-spectrum plane; then every warp
// takes kz columns of the plane and transforms them along y in registers, in
// place; finally the plane is stored contiguously (spec[c][x] is one n1*nh
// block). Inverse: load the half plane, inverse along y in place, then per
// pair of z rows the Hermitian spectra of both rows are combined, inverse-
// transformed in registers (real part row 2j, imaginary part row 2j+1) and
// added to DisGrad (same update as the separate inverse-z pass). No
// intermediate spectrum goes through global memory between the z and y
// transforms. Pairing rows of one component (instead of two components) keeps
// one plane per CTA: ~88 KB of shared memory in FP32 at 128^2, two CTAs per SM.

// Shared-memory row skew of the plane kernels: row r is stored at r + r/16.
// The warp FFTs scatter their outputs to rows k2 + E*brev5(lane), which
// without the skew fall on two 8-byte bank groups per half-warp (8-way
// conflicts); with it every half-warp access hits 16 distinct groups.
__device__ __forceinline__ int pskew(int r) { return r + (r >> 4); }
__host__ __device__ constexpr int plane_rows(int n) { return n + n / 16; }

template <typename T, int E>
__device__ __forceinline__ void plane_fwd_body(const PlaneArgs<T>& a, int bid, unsigned char* smem) {
    const Grid& g = a.g;
    const int n = g.n2, nh = g.nh, nhp = a.nhp;
    const int x = bid / 6, c = bid - 6 * x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    C2<T>* twz = reinterpret_cast<C2<T>*>(smem);
    C2<T>* twy = twz + n;
    C2<T>* S = twy + g.n1;
    C2<T>* R = S + (size_t)plane_rows(g.n1) * nhp + (size_t)warp * plane_rows(n);
    for (int i = threadIdx.x; i < n; i += blockDim.x) twz[i] = a.twz[i];
    for (int i = threadIdx.x; i < g.n1; i += blockDim.x) twy[i] = a.twy[i];
    __syncthreads();
    // one set of lane constants serves both axes (n1 == n2)
    WarpTw<T, E> wt;
    wt.init(twz, lane);
    const T* s0 = a.sig + (size_t)c * g.N + (size_t)x * g.n1 * n;
    const int npair = g.n1 / 2;
    // row pairs are software-pipelined: the next pair's loads are in flight
    // while the current pair is transformed
    C2<T> nxt[E];
    if (warp < npair)
#pragma unroll
        for (int q = 0; q < E; q++)
            nxt[q] = mk<T>(s0[(size_t)(2 * warp) * n + lane + 32 * q], s0[(size_t)(2 * warp + 1) * n + lane + 32 * q]);
    for (int j = warp; j < npair; j += PLANE_WARPS) {
        C2<T> v[E];
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = nxt[q];
        const int jn = j + PLANE_WARPS;
        if (jn < npair)
#pragma unroll
            for (int q = 0; q < E; q++)
                nxt[q] = mk<T>(s0[(size_t)(2 * jn) * n + lane + 32 * q], s0[(size_t)(2 * jn + 1) * n + lane + 32 * q]);
        warp_fft<T, E, -1>(v, wt);
        const int b = brev5(lane);
#pragma unroll
        for (int k2 = 0; k2 < E; k2++) R[pskew(k2 + E * b)] = v[k2];
        __syncwarp();
        C2<T>* r0 = S + (size_t)pskew(2 * j) * nhp;
        C2<T>* r1 = S + (size_t)pskew(2 * j + 1) * nhp;
        for (int k = lane; k < nh; k += 32) {
            const C2<T> z = R[pskew(k)];
            const C2<T> w = R[pskew(k == 0 ? 0 : n - k)];
            // row 2j: (Z(k) + conj Z(n-k))/2, row 2j+1: (Z(k) - conj Z(n-k))/(2i)
            r0[k] = mk<T>((T)0.5 * (z.x + w.x), (T)0.5 * (z.y - w.y));
            r1[k] = mk<T>((T)0.5 * (z.y + w.y), (T)-0.5 * (z.x - w.x));
        }
        __syncwarp();
    }
    __syncthreads();
    // y transforms of the n/2 + 1 columns as n/2 work items (a whole number per
    // warp): the columns kz = 0 and n/2 hold real values (the DC and Nyquist
    // terms of real rows), so one complex transform takes both, z = c0 + i cN,
    // and is split like the rows: C0 = (Z(k) + conj Z(-k))/2, CN = (Z(k) -
    // conj Z(-k))/(2i)
    for (int item = warp; item < nh - 1; item += PLANE_WARPS) {
        const int kz = item;
        C2<T> v[E];
        if (item == 0) {
#pragma unroll
            for (int q = 0; q < E; q++) {
                const int r = pskew(lane + 32 * q) * nhp;
                v[q] = mk<T>(S[r].x, S[r + nh - 1].x);
            }
        } else {
#pragma unroll
            for (int q = 0; q < E; q++) v[q] = S[pskew(lane + 32 * q) * nhp + kz];
        }
        warp_fft<T, E, -1>(v, wt);
        const int b = brev5(lane);
        if (item == 0) {
#pragma unroll
            for (int k2 = 0; k2 < E; k2++) R[pskew(k2 + E * b)] = v[k2];
            __syncwarp();
#pragma unroll
            for (int q = 0; q < E; q++) {
                const int k = lane + 32 * q;
                const C2<T> z = R[pskew(k)];
                const C2<T> w = R[pskew(k == 0 ? 0 : g.n1 - k)];
                const int r = pskew(k) * nhp;
                S[r] = mk<T>((T)0.5 * (z.x + w.x), (T)0.5 * (z.y - w.y));
                S[r + nh - 1] = mk<T>((T)0.5 * (z.y + w.y), (T)-0.5 * (z.x - w.x));
            }
            __syncwarp();
        } else {
#pragma unroll
            for (int k2 = 0; k2 < E; k2++) S[pskew(k2 + E * b) * nhp + kz] = v[k2];
        }
    }
    __syncthreads();
    C2<T>* o = a.spec + (size_t)c * g.Nh + (size_t)x * g.n1 * nh;
    for (int i = threadIdx.x; i < g.n1 * nh; i += blockDim.x) {
        const int y = a.dnh.div(i), k = i - y * nh;
        o[i] = S[pskew(y) * nhp + k];
    }
}

template <typename T, int E>
__device__ __forceinline__ void plane_inv_body(const PlaneArgs<T>& a, int bid, unsigned char* smem) {
    const Grid& g = a.g;
    const int n = g.n2, nh = g.nh, nhp = a.nhp;
    const int x = bid / a.nc, c = a.c0 + (bid - a.nc * x);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    C2<T>* twz = reinterpret_cast<C2<T>*>(smem);
    C2<T>* twy = twz + n;
    C2<T>* S = twy + g.n1;
    C2<T>* R = S + (size_t)plane_rows(g.n1) * nhp + (size_t)warp * plane_rows(n);
    for (int i = threadIdx.x; i < n; i += blockDim.x) twz[i] = a.twz[i];
    for (int i = threadIdx.x; i < g.n1; i += blockDim.x) twy[i] = a.twy[i];
    const C2<T>* in = a.spec + (size_t)c * g.Nh + (size_t)x * g.n1 * nh;
    for (int i = threadIdx.x; i < g.n1 * nh; i += blockDim.x) {
        const int y = a.dnh.div(i), k = i - y * nh;
        cp_async_elem<T>(S + pskew(y) * nhp + k, in + i);
    }
    // while the plane arrives: the deferred antisymmetric components of this
    // iteration into their sum, and their uniform correction (this pass runs
    // only in iterations whose correction is applied, while the X pass that
    // fills the pending buffer may run once more after the loop ended)
    if (a.acc) {
        const int ncta = a.nc * g.n0, nb = (a.ncommit + ncta - 1) / ncta;
        const int e0 = bid * nb, e1 = min(e0 + nb, a.ncommit);
        // CU elements per thread and round, all loads issued before the stores
        constexpr int CU = 4;
        for (int i0 = e0 + threadIdx.x; i0 < e1; i0 += CU * blockDim.x) {
            C2<T> s[CU], d[CU];
#pragma unroll
            for (int u = 0; u < CU; u++) {
                const int i = i0 + u * blockDim.x;
                if (i < e1) {
                    s[u] = a.acc[i];
                    d[u] = a.pend[i];
                }
            }
#pragma unroll
            for (int u = 0; u < CU; u++) {
                const int i = i0 + u * blockDim.x;
                if (i < e1) a.acc[i] = mk<T>(s[u].x + d[u].x, s[u].y + d[u].y);
            }
        }
        if (bid == 0 && threadIdx.x == 0)
#pragma unroll
            for (int q = 6; q < 9; q++) a.dE9_acc[q] += a.dE9[q];
    }
    cp_async_wait_all();
    __syncthreads();
    // one set of lane constants serves both axes (n1 == n2)
    WarpTw<T, E> wt;
    wt.init(twz, lane);
    // n/2 work items: the columns kz = 0 and n/2 are spectra of real rows
    // (Hermitian along y), so one complex inverse transform of C0 + i CN gives
    // both, c0 in the real and cN in the imaginary part
    for (int item = warp; item < nh - 1; item += PLANE_WARPS) {
        const int kz = item;
        C2<T> v[E];
        if (item == 0) {
#pragma unroll
            for (int q = 0; q < E; q++) {
                const int r = pskew(lane + 32 * q) * nhp;
                const C2<T> u = S[r], w = S[r + nh - 1];
                v[q] = mk<T>(u.x - w.y, u.y + w.x);
            }
        } else {
#pragma unroll
            for (int q = 0; q < E; q++) v[q] = S[pskew(lane + 32 * q) * nhp + kz];
        }
        warp_fft<T, E, 1>(v, wt);
        const int b = brev5(lane);
        if (item == 0) {
#pragma unroll
            for (int k2 = 0; k2 < E; k2++) {
                const int r = pskew(k2 + E * b) * nhp;
                S[r] = mk<T>(v[k2].x, (T)0);
                S[r + nh - 1] = mk<T>(v[k2].y, (T)0);
            }
        } else {
#pragma unroll
            for (int k2 = 0; k2 < E; k2++) S[pskew(k2 + E * b) * nhp + kz] = v[k2];
        }
    }
    __syncthreads();
    const T e = (T)a.dE9[c];
    const int npair = g.n1 / 2;
    for (int j = warp; j < npair; j += PLANE_WARPS) {
        T* d0 = a.dg + (size_t)c * g.N + ((size_t)x * g.n1 + 2 * j) * n;
        T* d1 = d0 + n;
        // DisGrad of the two rows, loaded before the transform hides its latency
        T p0[E], p1[E];
#pragma unroll
        for (int q = 0; q < E; q++) {
            p0[q] = d0[lane + 32 * q];
            p1[q] = d1[lane + 32 * q];
        }
        const C2<T>* r0 = S + (size_t)pskew(2 * j) * nhp;
        const C2<T>* r1 = S + (size_t)pskew(2 * j + 1) * nhp;
        C2<T> v[E];
#pragma unroll
        for (int q = 0; q < E; q++) {
            const int m = lane + 32 * q;
            const int mm = m < nh ? m : n - m;
            const C2<T> u = r0[mm];
            const C2<T> w = r1[mm];
            if (m < nh) v[q] = mk<T>(u.x - w.y, u.y + w.x);   // u + i w
            else v[q] = mk<T>(u.x + w.y, -u.y + w.x);         // conj u + i conj w
        }
        warp_fft<T, E, 1>(v, wt);
        const int b = brev5(lane);
#pragma unroll
        for (int k2 = 0; k2 < E; k2++) R[pskew(k2 + E * b)] = v[k2];
        __syncwarp();
#pragma unroll
        for (int q = 0; q < E; q++) {
            const int m = lane + 32 * q;
            const C2<T> z = R[pskew(m)];
            d0[m] = p0[q] + (e + z.x * a.invN);
            d1[m] = p1[q] + (e + z.y * a.invN);
        }
        __syncwarp();
    }
}

template <typename T, int E>
__global__ void __launch_bounds__(PLANE_THREADS, sizeof(T) == 4 ? PLANE_MIN_BLOCKS : 1) k_plane_fwd(const __grid_constant__ PlaneArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem[];
    if (!gate_open(a.macro, a.gate)) return;
    plane_fwd_body<T, E>(a, blockIdx.x, smem);
}

template <typename T, int E>
__global__ void __launch_bounds__(PLANE_THREADS, sizeof(T) == 4 ? PLANE_MIN_BLOCKS : 1) k_plane_inv(const __grid_constant__ PlaneArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem[];
    if (!gate_open(a.macro, a.gate)) return;
    plane_inv_body<T, E>(a, blockIdx.x, smem);
}

template <typename T, int E>
__global__ void __launch_bounds__(PLANE_THREADS, sizeof(T) == 4 ? PLANE_MIN_BLOCKS : 1) kb_plane_fwd(const PlaneArgs<T>* __restrict__ tab,
                                                              const int2* __restrict__ map) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int2 m = map[blockIdx.x];
    const PlaneArgs<T>& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    plane_fwd_body<T, E>(a, m.y, smem);
}

template <typename T, int E>
__global__ void __launch_bounds__(PLANE_THREADS, sizeof(T) == 4 ? PLANE_MIN_BLOCKS : 1) kb_plane_inv(const PlaneArgs<T>* __restrict__ tab,
                                                              const int2* __restrict__ map) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int2 m = map[blockIdx.x];
    const PlaneArgs<T>& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    plane_inv_body<T, E>(a, m.y, smem);
}

// ---- single-RVE kernels: arguments in the constant bank

template <typename T>
__global__ void __launch_bounds__(SPEC_THREADS) k_fwd_z(const __grid_constant__ ZArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem[];
    if (!gate_open(a.macro, a.gate)) return;
    fwd_z_body<T>(a, blockIdx.x, smem);
}

template <typename T, int SIGN>
__global__ void __launch_bounds__(SPEC_THREADS) k_y(const __grid_constant__ YArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem[];
    if (!gate_open(a.macro, a.gate)) return;
    y_body<T, SIGN>(a, blockIdx.x, smem);
}

template <typename T>
__global__ void __launch_bounds__(SPEC_THREADS) k_x_green(const __grid_constant__ XArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem[];
    if (!gate_open(a.macro, a.gate)) return;
    x_green_body<T, false>(a, a.gk, blockIdx.x, smem);
}

// Register budget of three CTAs per SM (80 registers, no spills): with the
// deferring form's six-row tile (56 KB) three CTAs fit an SM, 24 warps instead
// of 16 (X pass 0.061 -> 0.057 ms at 128^3; four CTAs at 64 registers spill).
template <typename T, int E>
__global__ void __launch_bounds__(XW_THREADS, 3) k_x_warp(const __grid_constant__ XArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem[];
    if (!gate_open(a.macro, a.gate)) return;
    x_warp_body<T, E, false>(a, a.gk, blockIdx.x, smem);
}

template <typename T>
__global__ void __launch_bounds__(SPEC_THREADS) k_inv_z(const __grid_constant__ ZArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem[];
    if (!gate_open(a.macro, a.gate)) return;
    inv_z_body<T>(a, blockIdx.x, smem);
}

// ---- batched kernels: one launch over many RVEs; map[b] = (RVE slot, CTA
// index within that RVE's grid), arguments of each RVE in a device table

template <typename T>
__global__ void __launch_bounds__(SPEC_THREADS) kb_fwd_z(const ZArgs<T>* __restrict__ tab,
                                                         const int2* __restrict__ map) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int2 m = map[blockIdx.x];
    const ZArgs<T>& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    fwd_z_body<T>(a, m.y, smem);
}

template <typename T, int SIGN>
__global__ void __launch_bounds__(SPEC_THREADS) kb_y(const YArgs<T>* __restrict__ tab,
                                                     const int2* __restrict__ map) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int2 m = map[blockIdx.x];
    const YArgs<T>& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    y_body<T, SIGN>(a, m.y, smem);
}

template <typename T>
__global__ void __launch_bounds__(SPEC_THREADS) kb_x_green(const XArgs<T>* __restrict__ tab,
                                                           const int2* __restrict__ map) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ GreenK<T> gks;
    const int2 m = map[blockIdx.x];
    const XArgs<T>& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    // C0 and S0 are contiguous (2 x 81 values)
    const T* src = &a.gk.c0[0][0][0][0];
    T* dst = &gks.c0[0][0][0][0];
    for (int i = threadIdx.x; i < 162; i += blockDim.x) dst[i] = src[i];
    if (threadIdx.x == 0) {
        gks.elast_bc = a.gk.elast_bc;
        gks.rn[0] = a.gk.rn[0];
        gks.rn[1] = a.gk.rn[1];
        gks.rn[2] = a.gk.rn[2];
    }
    __syncthreads();
    x_green_body<T, true>(a, gks, m.y, smem);
}

template <typename T, int E>
__global__ void __launch_bounds__(XW_THREADS, 3) kb_x_warp(const XArgs<T>* __restrict__ tab,
                                                      const int2* __restrict__ map) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ GreenK<T> gks;
    const int2 m = map[blockIdx.x];
    const XArgs<T>& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    const T* src = &a.gk.c0[0][0][0][0];
    T* dst = &gks.c0[0][0][0][0];
    for (int i = threadIdx.x; i < 162; i += blockDim.x) dst[i] = src[i];
    if (threadIdx.x == 0) {
        gks.elast_bc = a.gk.elast_bc;
        gks.rn[0] = a.gk.rn[0];
        gks.rn[1] = a.gk.rn[1];
        gks.rn[2] = a.gk.rn[2];
    }
    __syncthreads();
    x_warp_body<T, E, true>(a, gks, m.y, smem);
}

template <typename T>
__global__ void __launch_bounds__(SPEC_THREADS) kb_inv_z(const ZArgs<T>* __restrict__ tab,
                                                         const int2* __restrict__ map) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int2 m = map[blockIdx.x];
    const ZArgs<T>& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    inv_z_body<T>(a, m.y, smem);
}

// ------------------------------------------------------------ schedules

// Pencils per CTA that fit a shared-memory budget (at most 64).
static int pick_p(int per_pencil_elems, size_t elem, size_t budget) {
    const size_t per = (size_t)per_pencil_elems * elem;
    int p = (int)(budget / per);
    if (p < 1) p = 1;
    if (p > 64) p = 64;
    return p;
}

// Pencils per CTA: as many as the shared-memory budget allows, but few enough
// that the grid has at least `want` CTAs (a few per SM) to hide latency.
static int pencils(long long total_pencils, int pmax, long long want) {
    long long p = total_pencils / want;
    if (p > pmax) p = pmax;
    if (p < 1) p = 1;
    return (int)p;
}

constexpr size_t SPEC_BUDGET = 72 * 1024;
constexpr size_t SPEC_BUDGET_X = 75 * 1024;

// Largest pencil counts the shared-memory budgets and the register prefetch
// of the inverse-z pass allow, per pass (z, y, x).
void spec_pmax(const Grid& g, size_t es, int pmax[3]) {
    pmax[0] = pick_p(2 * z_pencil_stride(g.n2, es), es, SPEC_BUDGET);
    if (pmax[0] * g.n2 > SPEC_THREADS * INVZ_EPT) pmax[0] = (SPEC_THREADS * INVZ_EPT) / g.n2;
    if (pmax[0] < 1) pmax[0] = 1;
    pmax[1] = pick_p(2 * x_pencil_stride(g.n1, es), es, SPEC_BUDGET);
    if (pmax[1] > g.nh) pmax[1] = g.nh;
    pmax[2] = pick_p(18 * x_pencil_stride(g.n0, es), es, SPEC_BUDGET_X);
    if (pmax[2] > g.nh) pmax[2] = g.nh;
}

// Default pencils per CTA: the budget, reduced until the grid has 4 CTAs per SM.
void spec_default_p(const Grid& g, size_t es, int nsm, int P[3]) {
    int pmax[3];
    spec_pmax(g, es, pmax);
    const long long want = 4LL * nsm;
    P[0] = pencils((long long)g.n0 * g.n1, pmax[0], want);
    P[1] = pencils((long long)g.n0 * g.nh, pmax[1], want);
    P[2] = pencils((long long)g.n1 * g.nh, pmax[2], want);
}

template <typename T> static SpecSet<T>& spec_of(KernelSets& k);
template <> SpecSet<double>& spec_of<double>(KernelSets& k) { return k.s64; }
template <> SpecSet<float>& spec_of<float>(KernelSets& k) { return k.s32; }

// Launch arguments of the five spectral kernels for pencils-per-CTA P
// (z, y, x) and FFT plans pl (x, y, z); dg receives the inverse-z output.
constexpr size_t PLANE_SMEM_MAX = 200 * 1024;

// Elements per lane of the fused z+y passes for this grid (0: not eligible):
// n1 == n2 in {32, 64, 128} and the two planes fit in shared memory.
int plane_epl(const Grid& g, size_t elem) {
    if (g.n1 != g.n2) return 0;
    const int E = g.n2 / 32;
    if (E * 32 != g.n2 || (E != 1 && E != 2 && E != 4)) return 0;
    const int nhp = g.nh | 1;
    const size_t sm = (size_t)(g.n2 + g.n1 + plane_rows(g.n1) * nhp + PLANE_WARPS * plane_rows(g.n2)) * elem;
    return sm <= PLANE_SMEM_MAX ? E : 0;
}

// Index divisors of the z and y passes.
template <typename T> static void set_z_divisors(ZArgs<T>& za) {
    za.dn.set(za.g.n2);
    za.dnh.set(za.g.nh);
}
template <typename T> static void set_y_divisors(YArgs<T>& ya) {
    const int last = ya.g.nh - ((ya.g.nh + ya.P - 1) / ya.P - 1) * ya.P;
    ya.dnp[0].set(ya.P);
    ya.dnp[1].set(last);
}

// Index divisors of the X pass for its grid and pencils per CTA.
template <typename T> static void set_x_divisors(XArgs<T>& xa) {
    const Grid& g = xa.g;
    const int last = g.nh - ((g.nh + xa.P - 1) / xa.P - 1) * xa.P;
    xa.dn.set(g.n0);
    xa.dnp[0].set(xa.P);
    xa.dnnp[0].set(g.n0 * xa.P);
    xa.dnp[1].set(last);
    xa.dnnp[1].set(g.n0 * last);
    xa.dnh.set(g.nh);
}

template <typename T>
static void fill_spec_t(Ctx& c, SpecSet<T>& s, const int P[3], const FftPlan pl[3], T* sig, T* dg,
                        const C2<T>* const* tw, int fused, int xpass) {
    const Grid& g = c.g;
    C2<T>* spec = reinterpret_cast<C2<T>*>(c.spec);
    const size_t es = sizeof(C2<T>);
    ZArgs<T>& za = s.z;
    za.g = g; za.pl = pl[2]; za.macro = c.macro; za.gate = GATE_RUNNING; za.sig = sig; za.dg = dg;
    za.spec = spec; za.tw = tw[2]; za.dE9 = macro_field<double>(c.macro, offsetof(Macro, dE9));
    za.invN = (T)(1.0 / (double)g.N);
    za.P = P[0];
    const int ncol = g.n0 * g.n1;
    s.grid_z = (ncol + za.P - 1) / za.P;
    s.sm_z = (size_t)(g.n2 + 2 * za.P * z_pencil_stride(g.n2, es)) * es;
    set_z_divisors<T>(za);
    YArgs<T>& ya = s.yf;
    ya.g = g; ya.pl = pl[1]; ya.macro = c.macro; ya.gate = GATE_RUNNING; ya.spec = spec; ya.tw = tw[1];
    ya.ncomp = 6;
    ya.P = P[1];
    set_y_divisors<T>(ya);
    s.yi = ya;
    s.yi.ncomp = 9;
    s.grid_y = g.n0 * ((g.nh + ya.P - 1) / ya.P);
    s.sm_y = (size_t)(g.n1 + 2 * ya.P * x_pencil_stride(g.n1, es)) * es;
    XArgs<T>& xa = s.x;
    xa.g = g; xa.pl = pl[0]; xa.macro = c.macro; xa.gate = GATE_RUNNING; xa.spec = spec; xa.tw = tw[0];
    xa.P = P[2];
    const Material<T>& m = material_of<T>(c);
    for (int i = 0; i < 81; i++) {
        (&xa.gk.c0[0][0][0][0])[i] = (&m.c0[0][0][0][0])[i];
        (&xa.gk.s0[0][0][0][0])[i] = (&m.s0[0][0][0][0])[i];
    }
    xa.gk.elast_bc = m.elast_bc;
    xa.gk.rn[0] = (T)(1.0 / g.n0);
    xa.gk.rn[1] = (T)(1.0 / g.n1);
    xa.gk.rn[2] = (T)(1.0 / g.n2);
    set_x_divisors<T>(xa);
    s.grid_x = g.n1 * ((g.nh + xa.P - 1) / xa.P);
    s.sm_x = (size_t)(g.n0 + 18 * xa.P * x_pencil_stride(g.n0, es)) * es;
    // warp-register X pass: FP32 with n0 in {32, 64, 128}, unless switched off
    s.xw = (xpass != 0 && xw_eligible(g.n0, es)) ? g.n0 / 32 : 0;
    s.grid_xw = (g.n1 * g.nh + XW_PEN - 1) / XW_PEN;
    s.sm_xw = xw_smem(g.n0, es);
    s.epl = fused ? plane_epl(g, es) : 0;
    PlaneArgs<T>& pa = s.pl;
    pa.g = g; pa.macro = c.macro; pa.gate = GATE_RUNNING; pa.sig = sig; pa.dg = dg; pa.spec = spec;
    pa.twz = tw[2]; pa.twy = tw[1]; pa.dE9 = za.dE9; pa.invN = za.invN; pa.nhp = g.nh | 1;
    pa.dnh.set(g.nh);
    s.grid_pf = 6 * g.n0;
    s.sm_p = (size_t)(g.n2 + g.n1 + plane_rows(g.n1) * pa.nhp + PLANE_WARPS * plane_rows(g.n2)) * es;
    // FP32 with both warp-register passes: the antisymmetric components
    // (A12, A13, A23) of the correction feed nothing in the loop (the NR reads
    // the symmetric strain), so the X pass stores them untransformed, in its
    // lane order, to a pending buffer, the inverse plane pass adds that to
    // their running sum (a linear operation: the sum of the transforms is the
    // transform of the sum), and the sum is transformed once before the fold
    // at the end of the increment; their uniform part is summed in
    // Macro::dE9_acc. The X pass's tile then holds six components.
    s.defer = (sizeof(T) == 4 && s.xw && s.epl) ? 1 : 0;
    if (s.defer) s.sm_xw = xw_smem(g.n0, es, 6);
    double* acc9 = macro_field<double>(c.macro, offsetof(Macro, dE9_acc));
    C2<T>* acc = spec + 9 * (size_t)g.Nh;   // the sum, zeroed by the increment head
    C2<T>* pend = spec + 12 * (size_t)g.Nh; // this iteration's X pass output
    xa.mode = s.defer ? XM_DEFER : XM_ALL;
    xa.dbuf = s.defer ? pend : nullptr;
    pa.nc = s.defer ? 6 : 9;
    pa.c0 = 0;
    pa.dE9_acc = s.defer ? acc9 : nullptr;
    pa.acc = s.defer ? acc : nullptr;
    pa.pend = s.defer ? pend : nullptr;
    pa.ncommit = s.defer ? (int)(3 * (size_t)g.Nh) : 0;
    s.grid_pi = pa.nc * g.n0;
    s.xfl = xa;
    s.xfl.mode = XM_FLUSH;
    s.xfl.dbuf = s.defer ? acc : nullptr;
    s.pfl = pa;
    s.pfl.nc = 3;
    s.pfl.c0 = 6;
    s.pfl.dE9 = acc9;
    s.pfl.dE9_acc = nullptr;
    s.pfl.acc = nullptr;
    s.pfl.pend = nullptr;
    s.pfl.ncommit = 0;
    s.grid_pfl = 3 * g.n0;
}


template <typename T>
static void build_spec_t(Ctx& c, T* sig, T* dg, const C2<T>* const* tw) {
    int P[3];
    for (int a = 0; a < 3; a++) P[a] = c.sched_p[a];
    if (P[0] <= 0 || P[1] <= 0 || P[2] <= 0) {
        int d[3];
        spec_default_p(c.g, sizeof(C2<T>), c.nsm, d);
        for (int a = 0; a < 3; a++)
            if (P[a] <= 0) P[a] = d[a];
    }
    // fused z+y passes: FP32-bulk by default, FP64 only when chosen (tuner)
    const int fused = c.sched_fused < 0 ? (sizeof(T) == 4) : c.sched_fused;
    fill_spec_t<T>(c, spec_of<T>(*c.ks), P, c.pl, sig, dg, tw, fused, c.sched_xpass);
}

void build_spectral_sets(Ctx& c) {
    if (c.precision == 0) {
        const double2* tw[3] = {c.tw64[0], c.tw64[1], c.tw64[2]};
        build_spec_t<double>(c, c.sig64, c.dg64, tw);
    } else {
        const float2* tw[3] = {c.tw32[0], c.tw32[1], c.tw32[2]};
        build_spec_t<float>(c, c.sig32, c.ddg32, tw);
    }
}

template <typename T> static void spec_attributes() {
    const int mx = 227 * 1024;
    cudaFuncSetAttribute(k_fwd_z<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_inv_z<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_y<T, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_y<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_x_green<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx - 2048);
    cudaFuncSetAttribute(kb_fwd_z<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kb_inv_z<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kb_y<T, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kb_y<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kb_x_green<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx - 2048);
    if constexpr (sizeof(T) == 4) {  // the warp-register X pass is FP32 only
        cudaFuncSetAttribute(k_x_warp<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        cudaFuncSetAttribute(k_x_warp<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        cudaFuncSetAttribute(k_x_warp<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        cudaFuncSetAttribute(kb_x_warp<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx - 2048);
        cudaFuncSetAttribute(kb_x_warp<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx - 2048);
        cudaFuncSetAttribute(kb_x_warp<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx - 2048);
    }
    cudaFuncSetAttribute(k_plane_fwd<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_plane_fwd<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_plane_fwd<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_plane_inv<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_plane_inv<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_plane_inv<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kb_plane_fwd<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kb_plane_fwd<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kb_plane_fwd<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kb_plane_inv<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kb_plane_inv<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kb_plane_inv<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

template <typename T>
static void plane_launch(int fwd, int E, int grid, size_t sm, cudaStream_t st, const PlaneArgs<T>& a) {
    if (fwd) {
        if (E == 1) k_plane_fwd<T, 1><<<grid, PLANE_THREADS, sm, st>>>(a);
        else if (E == 2) k_plane_fwd<T, 2><<<grid, PLANE_THREADS, sm, st>>>(a);
        else k_plane_fwd<T, 4><<<grid, PLANE_THREADS, sm, st>>>(a);
    } else {
        if (E == 1) k_plane_inv<T, 1><<<grid, PLANE_THREADS, sm, st>>>(a);
        else if (E == 2) k_plane_inv<T, 2><<<grid, PLANE_THREADS, sm, st>>>(a);
        else k_plane_inv<T, 4><<<grid, PLANE_THREADS, sm, st>>>(a);
    }
}

template <typename T>
static void plane_launch_batch(int fwd, int E, const BatchLaunch& L, cudaStream_t st) {
    const PlaneArgs<T>* tab = (const PlaneArgs<T>*)L.tab;
    if (fwd) {
        if (E == 1) kb_plane_fwd<T, 1><<<L.nblk, PLANE_THREADS, L.smem, st>>>(tab, L.map);
        else if (E == 2) kb_plane_fwd<T, 2><<<L.nblk, PLANE_THREADS, L.smem, st>>>(tab, L.map);
        else kb_plane_fwd<T, 4><<<L.nblk, PLANE_THREADS, L.smem, st>>>(tab, L.map);
    } else {
        if (E == 1) kb_plane_inv<T, 1><<<L.nblk, PLANE_THREADS, L.smem, st>>>(tab, L.map);
        else if (E == 2) kb_plane_inv<T, 2><<<L.nblk, PLANE_THREADS, L.smem, st>>>(tab, L.map);
        else kb_plane_inv<T, 4><<<L.nblk, PLANE_THREADS, L.smem, st>>>(tab, L.map);
    }
}

// The X pass of the single-RVE chain: warp-register kernel when chosen.
template <typename T>
static void x_launch(const SpecSet<T>& s, const XArgs<T>& xa, cudaStream_t st) {
    if constexpr (sizeof(T) == 4) {
        if (s.xw == 1) k_x_warp<T, 1><<<s.grid_xw, XW_THREADS, s.sm_xw, st>>>(xa);
        else if (s.xw == 2) k_x_warp<T, 2><<<s.grid_xw, XW_THREADS, s.sm_xw, st>>>(xa);
        else if (s.xw == 4) k_x_warp<T, 4><<<s.grid_xw, XW_THREADS, s.sm_xw, st>>>(xa);
        if (s.xw) return;
    }
    k_x_green<T><<<s.grid_x, SPEC_THREADS, s.sm_x, st>>>(xa);
}

void spectral_attributes() {
    spec_attributes<double>();
    spec_attributes<float>();
}

// part: SPEC_ALL, SPEC_FWD (forward transforms and the X pass with the Green
// contraction: they write only the spectrum buffer) or SPEC_INV (inverse
// transforms with the DisGrad update).
template <typename T>
static cudaError_t spectral_t(Ctx& c, int gate, int part) {
    SpecSet<T>& s = spec_of<T>(*c.ks);
    ZArgs<T> za = s.z;
    YArgs<T> yf = s.yf, yi = s.yi;
    XArgs<T> xa = s.x;
    za.gate = yf.gate = yi.gate = xa.gate = gate;
    const bool fwd = part != SPEC_INV, inv = part != SPEC_FWD;
    if (s.epl) {
        PlaneArgs<T> pa = s.pl;
        pa.gate = gate;
        if (fwd) {
            prof_mark(c, PG_FWD_Z, true);
            plane_launch<T>(1, s.epl, s.grid_pf, s.sm_p, c.stream, pa);
            prof_mark(c, PG_FWD_Z, false);
            prof_mark(c, PG_X_GREEN, true);
            x_launch<T>(s, xa, c.stream);
            prof_mark(c, PG_X_GREEN, false);
        }
        if (inv) {
            prof_mark(c, PG_INV_Z, true);
            plane_launch<T>(0, s.epl, s.grid_pi, s.sm_p, c.stream, pa);
            prof_mark(c, PG_INV_Z, false);
        }
        return cudaGetLastError();
    }
    if (fwd) {
        prof_mark(c, PG_FWD_Z, true);
        k_fwd_z<T><<<s.grid_z, SPEC_THREADS, s.sm_z, c.stream>>>(za);
        prof_mark(c, PG_FWD_Z, false);
        prof_mark(c, PG_FWD_Y, true);
        k_y<T, -1><<<s.grid_y, SPEC_THREADS, s.sm_y, c.stream>>>(yf);
        prof_mark(c, PG_FWD_Y, false);
        prof_mark(c, PG_X_GREEN, true);
        x_launch<T>(s, xa, c.stream);
        prof_mark(c, PG_X_GREEN, false);
    }
    if (inv) {
        prof_mark(c, PG_INV_Y, true);
        k_y<T, 1><<<s.grid_y, SPEC_THREADS, s.sm_y, c.stream>>>(yi);
        prof_mark(c, PG_INV_Y, false);
        prof_mark(c, PG_INV_Z, true);
        k_inv_z<T><<<s.grid_z, SPEC_THREADS, s.sm_z, c.stream>>>(za);
        prof_mark(c, PG_INV_Z, false);
    }
    return cudaGetLastError();
}

cudaError_t launch_spectral(Ctx& c, int gate, int part) {
    return c.precision == 0 ? spectral_t<double>(c, gate, part) : spectral_t<float>(c, gate, part);
}

// End of the increment of a context that defers the antisymmetric part: its
// X pass flush and inverse plane pass over components 6..8 (before the fold).
template <typename T>
static cudaError_t flush_t(Ctx& c, int gate) {
    SpecSet<T>& s = spec_of<T>(*c.ks);
    if (!s.defer) return cudaSuccess;
    XArgs<T> xa = s.xfl;
    PlaneArgs<T> pa = s.pfl;
    xa.gate = pa.gate = gate;
    c.launches += 2;
    x_launch<T>(s, xa, c.stream);
    plane_launch<T>(0, s.epl, s.grid_pfl, s.sm_p, c.stream, pa);
    return cudaGetLastError();
}

cudaError_t launch_spectral_flush(Ctx& c, int gate) {
    return c.precision == 0 ? flush_t<double>(c, gate) : flush_t<float>(c, gate);
}

int spectral_flush_kernels(const Ctx& c) {
    return c.precision != 0 && c.ks->s32.defer ? 2 : 0;
}

// One pass of the spectral chain for a batch (see launch_spectral_batch).
template <typename T>
static int spectral_batch_t(const BatchLaunch* L, cudaStream_t st, int part) {
    const BatchLaunch &z = L[BL_Z], &yf = L[BL_YF], &x = L[BL_X], &yi = L[BL_YI];
    const int E[3] = {1, 2, 4};
    const bool fwd = part != SPEC_INV, inv = part != SPEC_FWD;
    int n = 0;
    for (int q = 0; q < 3 && fwd; q++)
        if (L[BL_PF1 + q].nblk) {
            plane_launch_batch<T>(1, E[q], L[BL_PF1 + q], st);
            n++;
        }
    if (fwd && z.nblk) {
        kb_fwd_z<T><<<z.nblk, SPEC_THREADS, z.smem, st>>>((const ZArgs<T>*)z.tab, z.map);
        kb_y<T, -1><<<yf.nblk, SPEC_THREADS, yf.smem, st>>>((const YArgs<T>*)yf.tab, yf.map);
        n += 2;
    }
    if constexpr (sizeof(T) == 4) {  // the warp-register X pass is FP32 only
        for (int q = 0; q < 3 && fwd; q++) {
            const BatchLaunch& w = L[BL_XW1 + q];
            if (!w.nblk) continue;
            const XArgs<T>* tab = (const XArgs<T>*)w.tab;
            if (q == 0) kb_x_warp<T, 1><<<w.nblk, XW_THREADS, w.smem, st>>>(tab, w.map);
            else if (q == 1) kb_x_warp<T, 2><<<w.nblk, XW_THREADS, w.smem, st>>>(tab, w.map);
            else kb_x_warp<T, 4><<<w.nblk, XW_THREADS, w.smem, st>>>(tab, w.map);
            n++;
        }
    }
    if (fwd && x.nblk) {
        kb_x_green<T><<<x.nblk, SPEC_THREADS, x.smem, st>>>((const XArgs<T>*)x.tab, x.map);
        n++;
    }
    if (inv && z.nblk) {
        kb_y<T, 1><<<yi.nblk, SPEC_THREADS, yi.smem, st>>>((const YArgs<T>*)yi.tab, yi.map);
        kb_inv_z<T><<<z.nblk, SPEC_THREADS, z.smem, st>>>((const ZArgs<T>*)z.tab, z.map);
        n += 2;
    }
    for (int q = 0; q < 3 && inv; q++)
        if (L[BL_PI1 + q].nblk) {
            plane_launch_batch<T>(0, E[q], L[BL_PI1 + q], st);
            n++;
        }
    return n;
}

int launch_spectral_batch(int precision, const BatchLaunch* L, cudaStream_t st, int part) {
    return precision == 0 ? spectral_batch_t<double>(L, st, part) : spectral_batch_t<float>(L, st, part);
}

// The flush of the slots that defer the antisymmetric part (FP32 only), per
// lane layout: X pass flush, then the inverse plane pass over components 6..8.
int launch_flush_batch(const BatchLaunch* L, cudaStream_t st) {
    const int E[3] = {1, 2, 4};
    int n = 0;
    for (int q = 0; q < 3; q++) {
        const BatchLaunch& w = L[BL_XFL1 + q];
        if (!w.nblk) continue;
        const XArgs<float>* tab = (const XArgs<float>*)w.tab;
        if (q == 0) kb_x_warp<float, 1><<<w.nblk, XW_THREADS, w.smem, st>>>(tab, w.map);
        else if (q == 1) kb_x_warp<float, 2><<<w.nblk, XW_THREADS, w.smem, st>>>(tab, w.map);
        else kb_x_warp<float, 4><<<w.nblk, XW_THREADS, w.smem, st>>>(tab, w.map);
        plane_launch_batch<float>(0, E[q], L[BL_PFL1 + q], st);
        n += 2;
    }
    return n;
}

// ------------------------------------------------------------- autotuner
//
// Per grid and precision: the FFT radix order of each axis and the pencils
// per CTA of each pass, chosen by timing the pass kernels on the context's
// own spectrum buffer (the inverse-z output goes to a scratch buffer, so the
// RVE state is untouched). Coordinate search: the radix orders with the
// current pencil count, then the pencil counts with the best order; passes
// are independent. Results are cached per (grid, precision) for the process.
// Pencil counts do not change the arithmetic; the radix order changes the
// FFT rounding only.

struct TuneEntry {
    int n0, n1, n2, prec;
    int P[3];
    FftPlan pl[3];
    int fused, xpass;
};
static std::mutex g_tune_mu;
static std::vector<TuneEntry> g_tune_cache;

static void plan_of(int n, const std::vector<int>& f, FftPlan& p) {
    memset(&p, 0, sizeof p);
    p.n = n;
    p.nf = (int)f.size();
    int ns = 1;
    for (int s = 0; s < p.nf; s++) {
        p.radix[s] = f[s];
        p.ns[s] = ns;
        ns *= f[s];
    }
    plan_divisors(p);
}

// Factor orders of n: radices 16 (with r16)/8/4/2 for the power-of-two part
// (at most one radix-2 stage), all distinct permutations, the odd factors
// after them or before them.
static std::vector<std::vector<int>> factor_orders(int n, bool r16) {
    int m = n, k = 0;
    while (m % 2 == 0) { m /= 2; k++; }
    std::vector<int> odd;
    for (int q : {3, 5})
        while (m % q == 0) { odd.push_back(q); m /= q; }
    for (int q = 7; m > 1; q += 2)
        while (m % q == 0) { odd.push_back(q); m /= q; }
    std::vector<std::vector<int>> out;
    // power-of-two part 2^k as radices 16/8/4 with at most one radix-2 stage
    for (int n16 = r16 ? k / 4 : 0; n16 >= 0; n16--)
        for (int n8 = (k - 4 * n16) / 3; n8 >= 0; n8--)
            for (int n2 = 0; n2 <= 1; n2++) {
                const int rest = k - 4 * n16 - 3 * n8 - n2;
                if (rest < 0 || rest % 2) continue;
                std::vector<int> f;
                for (int i = 0; i < n16; i++) f.push_back(16);
                for (int i = 0; i < n8; i++) f.push_back(8);
                for (int i = 0; i < rest / 2; i++) f.push_back(4);
                for (int i = 0; i < n2; i++) f.push_back(2);
                std::sort(f.begin(), f.end());
                do {
                    for (int front = 0; front < (odd.empty() ? 1 : 2); front++) {
                        std::vector<int> g;
                        if (front) g.insert(g.end(), odd.begin(), odd.end());
                        g.insert(g.end(), f.begin(), f.end());
                        if (!front) g.insert(g.end(), odd.begin(), odd.end());
                        if (g.size() <= 12 && std::find(out.begin(), out.end(), g) == out.end()) out.push_back(g);
                    }
                } while (std::next_permutation(f.begin(), f.end()) && out.size() < 64);
            }
    if (out.empty()) out.push_back(odd);
    return out;
}

constexpr size_t TUNE_SMEM_MAX = 200 * 1024;

// pass 0: z (forward + inverse), 1: y (forward + inverse), 2: x with the
// Green contraction, 3: fused z+y plane kernels (forward + inverse)
template <typename T>
static float time_pass(Ctx& c, int pass, const int P[3], const FftPlan pl[3], T* sig, T* scratch,
                       const C2<T>* const* tw, cudaEvent_t e0, cudaEvent_t e1, int xpass = 0) {
    SpecSet<T> s;
    fill_spec_t<T>(c, s, P, pl, sig, scratch, tw, pass == 3, xpass);
    s.z.gate = s.yf.gate = s.yi.gate = s.x.gate = s.pl.gate = GATE_ALWAYS;
    if (pass == 3 && !s.epl) return 1e30f;
    const size_t sm = pass == 0 ? s.sm_z : pass == 1 ? s.sm_y : pass == 2 ? (s.xw ? s.sm_xw : s.sm_x) : s.sm_p;
    if (sm > TUNE_SMEM_MAX) return 1e30f;
    if (pass == 0 && P[0] * c.g.n2 > SPEC_THREADS * INVZ_EPT) return 1e30f;
    auto launch = [&]() {
        if (pass == 3) {
            plane_launch<T>(1, s.epl, s.grid_pf, s.sm_p, c.stream, s.pl);
            plane_launch<T>(0, s.epl, s.grid_pi, s.sm_p, c.stream, s.pl);
        } else if (pass == 0) {
            k_fwd_z<T><<<s.grid_z, SPEC_THREADS, s.sm_z, c.stream>>>(s.z);
            k_inv_z<T><<<s.grid_z, SPEC_THREADS, s.sm_z, c.stream>>>(s.z);
        } else if (pass == 1) {
            k_y<T, -1><<<s.grid_y, SPEC_THREADS, s.sm_y, c.stream>>>(s.yf);
            k_y<T, 1><<<s.grid_y, SPEC_THREADS, s.sm_y, c.stream>>>(s.yi);
        } else {
            x_launch<T>(s, s.x, c.stream);
        }
    };
    launch();
    cudaEventRecord(e0, c.stream);
    const int reps = 5;
    for (int r = 0; r < reps; r++) launch();
    cudaEventRecord(e1, c.stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) return 1e30f;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return cudaGetLastError() == cudaSuccess ? ms / reps : 1e30f;
}

template <typename T>
static int tune_t(Ctx& c, T* sig, const C2<T>* const* tw, int force, double* gain) {
    const Grid& g = c.g;
    const int prec = c.precision;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        for (const TuneEntry& e : g_tune_cache)
            if (!force && e.n0 == g.n0 && e.n1 == g.n1 && e.n2 == g.n2 && e.prec == prec) {
                for (int a = 0; a < 3; a++) {
                    c.sched_p[a] = e.P[a];
                    c.pl[a] = e.pl[a];
                }
                c.sched_fused = e.fused;
                c.sched_xpass = e.xpass;
                build_sets(c);
                c.version++;
                if (gain) *gain = 0.0;
                return 0;
            }
    }
    T* scratch = nullptr;
    if (cudaMalloc((void**)&scratch, sizeof(T) * 9 * (size_t)g.N) != cudaSuccess) return 3;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int P[3];
    const SpecSet<T>& cur = spec_of<T>(*c.ks);
    P[0] = cur.z.P; P[1] = cur.yf.P; P[2] = cur.x.P;
    FftPlan pl[3] = {c.pl[0], c.pl[1], c.pl[2]};
    double t0 = 0.0, t1 = 0.0, tb[3] = {0.0, 0.0, 0.0};
    const int axis_of_pass[3] = {2, 1, 0};
    const int len_of_pass[3] = {g.n2, g.n1, g.n0};
    // the fused z+y kernels use the default radix-free warp transforms
    const float tf = time_pass<T>(c, 3, P, pl, sig, scratch, tw, e0, e1);
    const bool fused_default = cur.epl != 0;
    int xpass = 0;
    for (int pass = 0; pass < 3; pass++) {
        const int ax = axis_of_pass[pass];
        float best = time_pass<T>(c, pass, P, pl, sig, scratch, tw, e0, e1);
        if (pass == 2 && cur.xw) t0 += time_pass<T>(c, 2, P, pl, sig, scratch, tw, e0, e1, 1);
        else if (pass == 2 || !fused_default) t0 += best;
        // radix 16: FP32 X pass (the z and y passes are built without it)
        for (const std::vector<int>& f : factor_orders(len_of_pass[pass], sizeof(T) == 4 && pass == 2)) {
            FftPlan trial[3] = {pl[0], pl[1], pl[2]};
            plan_of(len_of_pass[pass], f, trial[ax]);
            const float t = time_pass<T>(c, pass, P, trial, sig, scratch, tw, e0, e1);
            if (t < best) {
                best = t;
                pl[ax] = trial[ax];
            }
        }
        const int cand[] = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64};
        for (int q : cand) {
            if (pass > 0 && q > g.nh) break;
            int Pt[3] = {P[0], P[1], P[2]};
            Pt[pass] = q;
            const float t = time_pass<T>(c, pass, Pt, pl, sig, scratch, tw, e0, e1);
            if (t < best) {
                best = t;
                P[pass] = q;
            }
        }
        if (pass == 2 && xw_eligible(g.n0, sizeof(C2<T>))) {
            // the warp-register X pass (no radix order or pencil count to choose)
            const float t = time_pass<T>(c, 2, P, pl, sig, scratch, tw, e0, e1, 1);
            if (t < best) {
                best = t;
                xpass = 1;
            }
        }
        tb[pass] = best;
    }
    if (fused_default) t0 += tf;
    const int fused = tf < tb[0] + tb[1] ? 1 : 0;
    t1 = (fused ? tf : tb[0] + tb[1]) + tb[2];
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamSynchronize(c.stream);
    cudaFree(scratch);
    if (cudaGetLastError() != cudaSuccess) return 2;
    for (int a = 0; a < 3; a++) {
        c.sched_p[a] = P[a];
        c.pl[a] = pl[a];
    }
    c.sched_fused = fused;
    c.sched_xpass = xpass;
    build_sets(c);
    c.version++;
    if (gain) *gain = t1 > 0 ? t0 / t1 : 0.0;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    TuneEntry e;
    e.n0 = g.n0; e.n1 = g.n1; e.n2 = g.n2; e.prec = prec;
    e.fused = fused;
    e.xpass = xpass;
    for (int a = 0; a < 3; a++) {
        e.P[a] = P[a];
        e.pl[a] = pl[a];
    }
    g_tune_cache.push_back(e);
    return 0;
}

int tune_spectral(Ctx& c, int force, double* gain) {
    cudaStreamSynchronize(c.stream);
    if (c.precision == 0) {
        const double2* tw[3] = {c.tw64[0], c.tw64[1], c.tw64[2]};
        return tune_t<double>(c, c.sig64, tw, force, gain);
    }
    const float2* tw[3] = {c.tw32[0], c.tw32[1], c.tw32[2]};
    return tune_t<float>(c, c.sig32, tw, force, gain);
}

}  // namespace evpg

// ---------------------------------------------------------------------------
// Allocation-free Green-operator correction.
//
// For callers that cannot allocate device memory on the call path -- code
// whose device memory is owned by another allocator (a framework's pool), or
// a service whose device footprint must be fixed when the library loads --
// this entry point runs the spectral chain of one equilibrium iteration on
// caller-owned input and output buffers. Its scratch (the nine half spectra,
// the twiddle tables and a zero macro correction) lives in
// the file-scope array below, which every GPU that loads the library holds
// until the process exits. Calls that overlap on the GPU share that array and
// race; callers serialise them (one stream, or events).

#include <math.h>
#include <string.h>

#include <mutex>

#include "evpg.h"

namespace evpg {

constexpr int NOALLOC_MAX_LEN = 64;               // per axis
constexpr long long NOALLOC_MAX_HALF = 32 * 32 * 17;  // n0*n1*(n2/2+1), e.g. 32^3
constexpr size_t NOALLOC_SPEC_BYTES = 9 * NOALLOC_MAX_HALF * sizeof(double2);
// twiddles of every axis length 1..NOALLOC_MAX_LEN, length n at entry n(n-1)/2
constexpr int NOALLOC_TW_ENTRIES = NOALLOC_MAX_LEN * (NOALLOC_MAX_LEN + 1) / 2;
constexpr size_t NOALLOC_TW_OFF = NOALLOC_SPEC_BYTES;
constexpr size_t NOALLOC_ZERO_OFF = NOALLOC_TW_OFF + ((NOALLOC_TW_ENTRIES * sizeof(double2) + 255) / 256) * 256;
constexpr size_t NOALLOC_BYTES = NOALLOC_ZERO_OFF + 256;  // 9 zero doubles, padded

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[128];  // device address of the array, per device

// Once per device, with that device current: look up the device address of
// the static array (its host-side name is not a device pointer) and write the
// twiddle tables of every axis length into it. Calls never overwrite them.
static int noalloc_setup(int dev, unsigned char** base) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return EVPG_ERR_CUDA;
        static double2 tw[NOALLOC_TW_ENTRIES];
        for (int n = 1; n <= NOALLOC_MAX_LEN; n++)
            for (int t = 0; t < n; t++) {
                double cc, ss;
                unit_root(t, n, &cc, &ss);
                tw[n * (n - 1) / 2 + t] = make_double2(cc, ss);
            }
        if (cudaMemcpy((unsigned char*)p + NOALLOC_TW_OFF, tw, sizeof tw, cudaMemcpyHostToDevice) != cudaSuccess)
            return EVPG_ERR_CUDA;
        g_noalloc_ptr[dev] = p;
    }
    *base = (unsigned char*)g_noalloc_ptr[dev];
    return EVPG_OK;
}

}  // namespace evpg

extern "C" int evpg_green_correction_noalloc(const double* sig6, double* du9, int32_t n0, int32_t n1,
                                             int32_t n2, const double c0[81], const double s0[81],
                                             int32_t elast_bc, void* stream) {
    using namespace evpg;
    const int n[3] = {n0, n1, n2};
    if (!sig6 || !du9 || !c0 || !s0) return EVPG_ERR_ARG;
    for (int a = 0; a < 3; a++)
        if (n[a] < 1 || n[a] > NOALLOC_MAX_LEN) return EVPG_ERR_ARG;
    const long long half = (long long)n0 * n1 * (n2 / 2 + 1);
    if (half > NOALLOC_MAX_HALF) return EVPG_ERR_ARG;  // beyond the static scratch
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return EVPG_ERR_CUDA;
    unsigned char* base = nullptr;
    if (noalloc_setup(dev, &base) != EVPG_OK) return EVPG_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    Grid g;
    g.n0 = n0; g.n1 = n1; g.n2 = n2; g.nh = n2 / 2 + 1; g.N = n0 * n1 * n2; g.Nh = half;
    FftPlan pl[3];
    for (int a = 0; a < 3; a++) make_plan(n[a], pl[a]);
    double2* spec = (double2*)base;
    const double2* twd = (const double2*)(base + NOALLOC_TW_OFF);
    double* zero9 = (double*)(base + NOALLOC_ZERO_OFF + 16);
    const double2* twp[3] = {twd + n0 * (n0 - 1) / 2, twd + n1 * (n1 - 1) / 2, twd + n2 * (n2 - 1) / 2};
    // the macro correction must read zero; the output is accumulated into,
    // so it starts at zero too
    if (cudaMemsetAsync(base + NOALLOC_ZERO_OFF, 0, 256, st) != cudaSuccess) return EVPG_ERR_CUDA;
    if (cudaMemsetAsync(du9, 0, (size_t)9 * g.N * sizeof(double), st) != cudaSuccess) return EVPG_ERR_CUDA;

    const size_t es = sizeof(double2), budget = 72 * 1024;
    ZArgs<double> za;
    za.g = g; za.pl = pl[2]; za.macro = nullptr; za.gate = GATE_ALWAYS; za.sig = sig6; za.dg = du9; za.spec = spec;
    za.tw = twp[2]; za.dE9 = zero9; za.invN = 1.0 / (double)g.N;
    za.P = pick_p(2 * z_pencil_stride(n2, es), es, budget);
    if (za.P * n2 > SPEC_THREADS * INVZ_EPT) za.P = (SPEC_THREADS * INVZ_EPT) / n2;
    set_z_divisors<double>(za);
    const int ncol = n0 * n1;
    const size_t sm = (size_t)(n2 + 2 * za.P * z_pencil_stride(n2, es)) * es;
    YArgs<double> ya;
    ya.g = g; ya.pl = pl[1]; ya.macro = nullptr; ya.gate = GATE_ALWAYS; ya.spec = spec; ya.tw = twp[1]; ya.ncomp = 6;
    ya.P = pick_p(2 * x_pencil_stride(n1, es), es, budget);
    if (ya.P > g.nh) ya.P = g.nh;
    set_y_divisors<double>(ya);
    const size_t smy = (size_t)(n1 + 2 * ya.P * x_pencil_stride(n1, es)) * es;
    const int ntile_y = (g.nh + ya.P - 1) / ya.P;
    XArgs<double> xa;
    xa.g = g; xa.pl = pl[0]; xa.macro = nullptr; xa.gate = GATE_ALWAYS; xa.spec = spec; xa.tw = twp[0];
    xa.mode = XM_ALL; xa.dbuf = nullptr;
    xa.P = pick_p(18 * x_pencil_stride(n0, es), es, 150 * 1024);
    if (xa.P > g.nh) xa.P = g.nh;
    for (int i = 0; i < 81; i++) {
        (&xa.gk.c0[0][0][0][0])[i] = c0[i];
        (&xa.gk.s0[0][0][0][0])[i] = s0[i];
    }
    xa.gk.elast_bc = elast_bc;
    xa.gk.rn[0] = 1.0 / n0;
    xa.gk.rn[1] = 1.0 / n1;
    xa.gk.rn[2] = 1.0 / n2;
    set_x_divisors<double>(xa);
    const size_t smx = (size_t)(n0 + 18 * xa.P * x_pencil_stride(n0, es)) * es;
    const int ntile_x = (g.nh + xa.P - 1) / xa.P;
    set_kernel_attributes();
    k_fwd_z<double><<<(ncol + za.P - 1) / za.P, SPEC_THREADS, sm, st>>>(za);
    k_y<double, -1><<<n0 * ntile_y, SPEC_THREADS, smy, st>>>(ya);
    k_x_green<double><<<n1 * ntile_x, SPEC_THREADS, smx, st>>>(xa);
    ya.ncomp = 9;
    k_y<double, 1><<<n0 * ntile_y, SPEC_THREADS, smy, st>>>(ya);
    k_inv_z<double><<<(ncol + za.P - 1) / za.P, SPEC_THREADS, sm, st>>>(za);
    return cudaGetLastError() == cudaSuccess ? EVPG_OK : EVPG_ERR_CUDA;
}
