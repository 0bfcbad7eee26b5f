// Spectral-chain kernels (see evpg_spectral.cuh) and their launcher.
#include "evpg_ctx.h"
#include "evpg_spectral.cuh"

namespace evpg {

template <typename T> struct GreenK {
    T c0[3][3][3][3];
    T s0[3][3][3][3];
    int elast_bc;
};

template <typename T> struct ZArgs {
    Grid g;
    FftPlan pl;
    const int* done;
    const T* sig;        // [6][N] real
    T* dg;               // [9][N] real (inverse pass)
    C2<T>* spec;         // [9][Nh]
    const C2<T>* tw;
    const double* dE9;   // macro correction added in the inverse pass
    int P;
    T invN;
};

template <typename T> struct YArgs {
    Grid g;
    FftPlan pl;
    const int* done;
    C2<T>* spec;
    const C2<T>* tw;
    int ncomp, P;
};

template <typename T> struct XArgs {
    Grid g;
    FftPlan pl;
    const int* done;
    C2<T>* spec;
    const C2<T>* tw;
    int P;
    GreenK<T> gk;
};

template <typename T>
__device__ __forceinline__ void load_tw(C2<T>* tw, const C2<T>* src, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) tw[i] = src[i];
}

// Forward z: three complex FFTs of (sig[2p] + i sig[2p+1]) per column, split
// into the two half spectra.
template <typename T>
__global__ void __launch_bounds__(256) k_fwd_z(const __grid_constant__ ZArgs<T> a) {
    if (*a.done) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid& g = a.g;
    const int n = g.n2, nh = g.nh, P = a.P;
    C2<T>* tw = reinterpret_cast<C2<T>*>(smem);
    C2<T>* bA = tw + n;
    C2<T>* bB = bA + P * n;
    const int ncol = g.n0 * g.n1, c0 = blockIdx.x * P, np = min(P, ncol - c0);
    load_tw<T>(tw, a.tw, n);
    for (int pair = 0; pair < 3; pair++) {
        const T* sa = a.sig + (size_t)(2 * pair) * g.N + (size_t)c0 * n;
        const T* sb = a.sig + (size_t)(2 * pair + 1) * g.N + (size_t)c0 * n;
        for (int i = threadIdx.x; i < np * n; i += blockDim.x) bA[i] = mk<T>(sa[i], sb[i]);
        __syncthreads();
        const C2<T>* r = fft_batch<T, -1>(bA, bB, np, n, a.pl, tw);
        C2<T>* oa = a.spec + (size_t)(2 * pair) * g.Nh + (size_t)c0 * nh;
        C2<T>* ob = a.spec + (size_t)(2 * pair + 1) * g.Nh + (size_t)c0 * nh;
        for (int i = threadIdx.x; i < np * nh; i += blockDim.x) {
            const int col = i / nh, k = i - col * nh;
            const C2<T> z = r[col * n + k];
            const C2<T> w = r[col * n + (k == 0 ? 0 : n - k)];
            // A = (Z(k) + conj Z(n-k))/2, B = (Z(k) - conj Z(n-k))/(2i)
            oa[i] = mk<T>((T)0.5 * (z.x + w.x), (T)0.5 * (z.y - w.y));
            ob[i] = mk<T>((T)0.5 * (z.y + w.y), (T)-0.5 * (z.x - w.x));
        }
        __syncthreads();
    }
}

// c2c along y on ncomp planes, pencils (x, kz..kz+P).
template <typename T, int SIGN>
__global__ void __launch_bounds__(256) k_y(const __grid_constant__ YArgs<T> a) {
    if (*a.done) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid& g = a.g;
    const int n = g.n1, ps = n + 1, P = a.P, nh = g.nh;
    C2<T>* tw = reinterpret_cast<C2<T>*>(smem);
    C2<T>* bA = tw + n;
    C2<T>* bB = bA + P * ps;
    const int ntile = (nh + P - 1) / P;
    const int x = blockIdx.x / ntile, kz0 = (blockIdx.x % ntile) * P, np = min(P, nh - kz0);
    load_tw<T>(tw, a.tw, n);
    for (int c = 0; c < a.ncomp; c++) {
        C2<T>* base = a.spec + (size_t)c * g.Nh + (size_t)x * n * nh + kz0;
        for (int i = threadIdx.x; i < n * np; i += blockDim.x) {
            const int y = i / np, kk = i - y * np;
            bA[kk * ps + y] = base[(size_t)y * nh + kk];
        }
        __syncthreads();
        const C2<T>* r = fft_batch<T, SIGN>(bA, bB, np, ps, a.pl, tw);
        for (int i = threadIdx.x; i < n * np; i += blockDim.x) {
            const int y = i / np, kk = i - y * np;
            base[(size_t)y * nh + kk] = r[kk * ps + y];
        }
        __syncthreads();
    }
}

// Forward x, Green contraction, inverse x on pencils (y, kz..kz+P).
template <typename T>
__global__ void __launch_bounds__(256) k_x_green(const __grid_constant__ XArgs<T> a) {
    if (*a.done) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid& g = a.g;
    const int n = g.n0, ps = n + 1, P = a.P, nh = g.nh;
    C2<T>* tw = reinterpret_cast<C2<T>*>(smem);
    C2<T>* bA = tw + n;
    C2<T>* bB = bA + 9 * P * ps;
    const int ntile = (nh + P - 1) / P;
    const int y = blockIdx.x / ntile, kz0 = (blockIdx.x % ntile) * P, np = min(P, nh - kz0);
    const size_t xs = (size_t)g.n1 * nh;
    load_tw<T>(tw, a.tw, n);
    for (int i = threadIdx.x; i < 6 * n * np; i += blockDim.x) {
        const int c = i / (n * np), rem = i - c * n * np, x = rem / np, kk = rem - x * np;
        bA[(c * np + kk) * ps + x] = a.spec[(size_t)c * g.Nh + x * xs + (size_t)y * nh + kz0 + kk];
    }
    __syncthreads();
    C2<T>* R = fft_batch<T, -1>(bA, bB, 6 * np, ps, a.pl, tw);
    C2<T>* W = (R == bA) ? bB : bA;
    for (int i = threadIdx.x; i < n * np; i += blockDim.x) {
        const int kk = i / n, kx = i - kk * n, kz = kz0 + kk, ky = y;
        C2<T> sb[6], du[9];
#pragma unroll
        for (int c = 0; c < 6; c++) sb[c] = R[(c * np + kk) * ps + kx];
        if ((kx | ky | kz) == 0) {
            green_k0<T>(a.gk.s0, a.gk.elast_bc, sb, du);
        } else {
            T nv[3];
            kvec<T>(kx, ky, kz, g, nv);
            green_du<T>(a.gk.c0, nv, sb, du);
            const bool nyq = ((g.n0 & 1) == 0 && 2 * kx == g.n0) ||
                             ((g.n1 & 1) == 0 && 2 * ky == g.n1) ||
                             ((g.n2 & 1) == 0 && 2 * kz == g.n2);
            if (nyq) {
                // Hermitian part: (du(k) + conj du(-k))/2 with sig_hat(-k) = conj sig_hat(k)
                C2<T> sm[6], dm[9];
#pragma unroll
                for (int c = 0; c < 6; c++) sm[c] = cconj<T>(sb[c]);
                const int mx = (g.n0 - kx) % g.n0, my = (g.n1 - ky) % g.n1, mz = (g.n2 - kz) % g.n2;
                kvec<T>(mx, my, mz, g, nv);
                green_du<T>(a.gk.c0, nv, sm, dm);
#pragma unroll
                for (int c = 0; c < 9; c++)
                    du[c] = mk<T>((T)0.5 * (du[c].x + dm[c].x), (T)0.5 * (du[c].y - dm[c].y));
            }
        }
#pragma unroll
        for (int c = 0; c < 9; c++) W[(c * np + kk) * ps + kx] = du[c];
    }
    __syncthreads();
    const C2<T>* R2 = fft_batch<T, 1>(W, (W == bA) ? bB : bA, 9 * np, ps, a.pl, tw);
    for (int i = threadIdx.x; i < 9 * n * np; i += blockDim.x) {
        const int c = i / (n * np), rem = i - c * n * np, x = rem / np, kk = rem - x * np;
        a.spec[(size_t)c * g.Nh + x * xs + (size_t)y * nh + kz0 + kk] = R2[(c * np + kk) * ps + x];
    }
}

// Inverse z: pairs of Hermitian half spectra -> one complex IFFT -> two real
// fields; DisGrad += dE + re/N (evolution.c:1197). The DisGrad values of a
// pair are loaded into registers before its transform, so their latency
// overlaps the FFT stages (at most INVZ_EPT elements per thread).
constexpr int INVZ_EPT = 16;

template <typename T>
__global__ void __launch_bounds__(256) k_inv_z(const __grid_constant__ ZArgs<T> a) {
    if (*a.done) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid& g = a.g;
    const int n = g.n2, nh = g.nh, P = a.P;
    C2<T>* tw = reinterpret_cast<C2<T>*>(smem);
    C2<T>* bA = tw + n;
    C2<T>* bB = bA + P * n;
    const int ncol = g.n0 * g.n1, c0 = blockIdx.x * P, np = min(P, ncol - c0);
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
            const int col = i / n, k = i - col * n;
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
            bA[i] = z;
        }
        __syncthreads();
        const C2<T>* r = fft_batch<T, 1>(bA, bB, np, n, a.pl, tw);
        const T ea = (T)a.dE9[ca], eb = hasb ? (T)a.dE9[cb] : (T)0;
#pragma unroll
        for (int e = 0; e < INVZ_EPT; e++) {
            const int i = threadIdx.x + e * blockDim.x;
            if (i < tot) {
                const C2<T> z = r[i];
                da[i] = pa[e] + (ea + z.x * a.invN);
                if (hasb) db[i] = pb[e] + (eb + z.y * a.invN);
            }
        }
        __syncthreads();
    }
}

template <typename T> static int pick_p(int n, int per_pencil_elems, size_t elem, size_t budget) {
    const size_t per = (size_t)per_pencil_elems * elem;
    int p = (int)(budget / per);
    if (p < 1) p = 1;
    if (p > 64) p = 64;
    (void)n;
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

template <typename T>
static cudaError_t spectral_t(Ctx& c, T* sig, T* dg, const C2<T>* const* tw) {
    const Grid& g = c.g;
    C2<T>* spec = reinterpret_cast<C2<T>*>(c.spec);
    const int* done = macro_field<int>(c.macro, offsetof(Macro, done));
    const size_t es = sizeof(C2<T>);
    const size_t budget = 72 * 1024;
    int nsm = 152;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    }
    const long long want = 4LL * nsm;
    cudaError_t e;
    {
        ZArgs<T> za;
        za.g = g; za.pl = c.pl[2]; za.done = done; za.sig = sig; za.dg = dg; za.spec = spec;
        za.tw = tw[2]; za.dE9 = macro_field<double>(c.macro, offsetof(Macro, dE9));
        za.invN = (T)(1.0 / (double)g.N);
        const int ncol = g.n0 * g.n1;
        za.P = pencils(ncol, pick_p<T>(g.n2, 2 * g.n2, es, budget), want);
        if (za.P * g.n2 > 256 * INVZ_EPT) za.P = (256 * INVZ_EPT) / g.n2;
        if (za.P < 1) za.P = 1;
        const size_t sm = (size_t)(g.n2 + 2 * za.P * g.n2) * es;
        cudaFuncSetAttribute(k_fwd_z<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        cudaFuncSetAttribute(k_inv_z<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        prof_mark(c, PG_FWD_Z, true);
        k_fwd_z<T><<<(ncol + za.P - 1) / za.P, 256, sm, c.stream>>>(za);
        prof_mark(c, PG_FWD_Z, false);
        // y forward
        YArgs<T> ya;
        ya.g = g; ya.pl = c.pl[1]; ya.done = done; ya.spec = spec; ya.tw = tw[1]; ya.ncomp = 6;
        ya.P = pencils((long long)g.n0 * g.nh, pick_p<T>(g.n1, 2 * (g.n1 + 1), es, budget), want);
        if (ya.P > g.nh) ya.P = g.nh;
        const size_t smy = (size_t)(g.n1 + 2 * ya.P * (g.n1 + 1)) * es;
        cudaFuncSetAttribute(k_y<T, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smy);
        cudaFuncSetAttribute(k_y<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smy);
        const int ntile_y = (g.nh + ya.P - 1) / ya.P;
        prof_mark(c, PG_FWD_Y, true);
        k_y<T, -1><<<g.n0 * ntile_y, 256, smy, c.stream>>>(ya);
        prof_mark(c, PG_FWD_Y, false);
        // x + Green
        XArgs<T> xa;
        xa.g = g; xa.pl = c.pl[0]; xa.done = done; xa.spec = spec; xa.tw = tw[0];
        xa.P = pencils((long long)g.n1 * g.nh, pick_p<T>(g.n0, 18 * (g.n0 + 1), es, 75 * 1024), want);
        if (xa.P > g.nh) xa.P = g.nh;
        const Material<T>& m = material_of<T>(c);
        for (int i = 0; i < 81; i++) {
            (&xa.gk.c0[0][0][0][0])[i] = (&m.c0[0][0][0][0])[i];
            (&xa.gk.s0[0][0][0][0])[i] = (&m.s0[0][0][0][0])[i];
        }
        xa.gk.elast_bc = m.elast_bc;
        const size_t smx = (size_t)(g.n0 + 18 * xa.P * (g.n0 + 1)) * es;
        cudaFuncSetAttribute(k_x_green<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx);
        const int ntile_x = (g.nh + xa.P - 1) / xa.P;
        prof_mark(c, PG_X_GREEN, true);
        k_x_green<T><<<g.n1 * ntile_x, 256, smx, c.stream>>>(xa);
        prof_mark(c, PG_X_GREEN, false);
        // y inverse
        ya.ncomp = 9;
        prof_mark(c, PG_INV_Y, true);
        k_y<T, 1><<<g.n0 * ntile_y, 256, smy, c.stream>>>(ya);
        prof_mark(c, PG_INV_Y, false);
        prof_mark(c, PG_INV_Z, true);
        k_inv_z<T><<<(ncol + za.P - 1) / za.P, 256, sm, c.stream>>>(za);
        prof_mark(c, PG_INV_Z, false);
    }
    e = cudaGetLastError();
    return e;
}

cudaError_t launch_spectral(Ctx& c) {
    if (c.precision == 0) {
        const double2* tw[3] = {c.tw64[0], c.tw64[1], c.tw64[2]};
        return spectral_t<double>(c, c.sig64, c.dg64, tw);
    }
    const float2* tw[3] = {c.tw32[0], c.tw32[1], c.tw32[2]};
    return spectral_t<float>(c, c.sig32, c.ddg32, tw);
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
// the twiddle tables, a zero loop flag and a zero macro correction) lives in
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
constexpr size_t NOALLOC_TW_OFF = NOALLOC_SPEC_BYTES;
constexpr size_t NOALLOC_ZERO_OFF = NOALLOC_TW_OFF + 3 * NOALLOC_MAX_LEN * sizeof(double2);
constexpr size_t NOALLOC_BYTES = NOALLOC_ZERO_OFF + 256;  // flag (int) + 9 doubles, padded

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[128];  // device address of the array, per device

static void na_plan(int n, FftPlan& p) {
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
}

// exp(-2 pi i t/n) with exact axis values (same table as the context path)
static double2 na_root(long t, long n) {
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
    return make_double2((double)cc, -(double)ss);
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
    unsigned char* base;
    {
        // once per device, with that device current: the device address of the
        // static array (its host-side name is not a device pointer)
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return EVPG_ERR_CUDA;
            g_noalloc_ptr[dev] = p;
        }
        base = (unsigned char*)g_noalloc_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    Grid g;
    g.n0 = n0; g.n1 = n1; g.n2 = n2; g.nh = n2 / 2 + 1; g.N = n0 * n1 * n2; g.Nh = half;
    FftPlan pl[3];
    double2 tw[3][NOALLOC_MAX_LEN];
    for (int a = 0; a < 3; a++) {
        na_plan(n[a], pl[a]);
        for (int t = 0; t < n[a]; t++) tw[a][t] = na_root(t, n[a]);
    }
    double2* spec = (double2*)base;
    double2* twd = (double2*)(base + NOALLOC_TW_OFF);
    int* zero_flag = (int*)(base + NOALLOC_ZERO_OFF);
    double* zero9 = (double*)(base + NOALLOC_ZERO_OFF + 16);
    const double2* twp[3] = {twd, twd + NOALLOC_MAX_LEN, twd + 2 * NOALLOC_MAX_LEN};
    // the loop flag and the macro correction must read zero; the output is
    // accumulated into, so it starts at zero too
    if (cudaMemsetAsync(base + NOALLOC_ZERO_OFF, 0, 256, st) != cudaSuccess) return EVPG_ERR_CUDA;
    if (cudaMemsetAsync(du9, 0, (size_t)9 * g.N * sizeof(double), st) != cudaSuccess) return EVPG_ERR_CUDA;
    if (cudaMemcpyAsync(twd, tw, sizeof tw, cudaMemcpyHostToDevice, st) != cudaSuccess) return EVPG_ERR_CUDA;

    const size_t es = sizeof(double2), budget = 72 * 1024;
    ZArgs<double> za;
    za.g = g; za.pl = pl[2]; za.done = zero_flag; za.sig = sig6; za.dg = du9; za.spec = spec;
    za.tw = twp[2]; za.dE9 = zero9; za.invN = 1.0 / (double)g.N;
    za.P = pick_p<double>(n2, 2 * n2, es, budget);
    if (za.P * n2 > 256 * INVZ_EPT) za.P = (256 * INVZ_EPT) / n2;
    const int ncol = n0 * n1;
    const size_t sm = (size_t)(n2 + 2 * za.P * n2) * es;
    YArgs<double> ya;
    ya.g = g; ya.pl = pl[1]; ya.done = zero_flag; ya.spec = spec; ya.tw = twp[1]; ya.ncomp = 6;
    ya.P = pick_p<double>(n1, 2 * (n1 + 1), es, budget);
    if (ya.P > g.nh) ya.P = g.nh;
    const size_t smy = (size_t)(n1 + 2 * ya.P * (n1 + 1)) * es;
    const int ntile_y = (g.nh + ya.P - 1) / ya.P;
    XArgs<double> xa;
    xa.g = g; xa.pl = pl[0]; xa.done = zero_flag; xa.spec = spec; xa.tw = twp[0];
    xa.P = pick_p<double>(n0, 18 * (n0 + 1), es, 150 * 1024);
    if (xa.P > g.nh) xa.P = g.nh;
    for (int i = 0; i < 81; i++) {
        (&xa.gk.c0[0][0][0][0])[i] = c0[i];
        (&xa.gk.s0[0][0][0][0])[i] = s0[i];
    }
    xa.gk.elast_bc = elast_bc;
    const size_t smx = (size_t)(n0 + 18 * xa.P * (n0 + 1)) * es;
    const int ntile_x = (g.nh + xa.P - 1) / xa.P;
    cudaFuncSetAttribute(k_fwd_z<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaFuncSetAttribute(k_inv_z<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaFuncSetAttribute(k_y<double, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smy);
    cudaFuncSetAttribute(k_y<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smy);
    cudaFuncSetAttribute(k_x_green<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx);
    k_fwd_z<double><<<(ncol + za.P - 1) / za.P, 256, sm, st>>>(za);
    k_y<double, -1><<<n0 * ntile_y, 256, smy, st>>>(ya);
    k_x_green<double><<<n1 * ntile_x, 256, smx, st>>>(xa);
    ya.ncomp = 9;
    k_y<double, 1><<<n0 * ntile_y, 256, smy, st>>>(ya);
    k_inv_z<double><<<(ncol + za.P - 1) / za.P, 256, sm, st>>>(za);
    return cudaGetLastError() == cudaSuccess ? EVPG_OK : EVPG_ERR_CUDA;
}
