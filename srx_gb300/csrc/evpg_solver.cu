// Per-voxel kernels of the equilibrium iteration and of the increment head
// and tail, plus the device-side macro update.
//
//   k_nr         UpdateStress (evolution.c:157-427) with StrainRate_Orowan
//                (constitutive.c:507-728): Newton on
//                R(s) = s - lambda + C066 (Eps + edot(s) dt + S s - eps)
//                one thread per voxel. The Newton step J^-1 R with
//                J = I + C066 (S + dt d_edot) is computed as
//                M^-1 (S066 R), M = S066 + S + dt d_edot (C066 S066 = I), which
//                is symmetric positive definite, so an unpivoted LDL^T
//                suffices. Plain update or the NR_MODIFIED line search.
//   k_macro      error Allreduce + get_smacro + normalisation + loop test
//                (evolution.c:1227-1252, 590-664), one CTA, FP64.
//   k_begin      increment head: VelGrad <- DisGrad, DisGrad += Udot dt,
//                update_schmid, flow-rule constants of this increment.
//   k_end        increment tail: VelGrad, Eps, update_orient,
//                DislocationEvolution, partial sums of the averages.
//   k_end_reduce AvgDislocation and the Eps/Edot averages.
#include "evpg_ctx.h"

#include <stdio.h>

namespace evpg {


// ------------------------------------------------------------ reductions

// Compensated (two-sum) accumulation, used for FP32 partials.
struct KSum {
    float s, c;
    __device__ __forceinline__ void add(float x) {
        const float t = s + x;
        const float bp = t - s;
        c += (s - (t - bp)) + (x - bp);
        s = t;
    }
};

template <int NQ>
__device__ __forceinline__ void block_reduce_store(double (&v)[NQ], double* out) {
    __shared__ double red[NQ][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        double x = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[q][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < NQ) {
        double s = 0.0;
        for (int w = 0; w < nw; w++) s += red[threadIdx.x][w];
        out[threadIdx.x] = s;
    }
}

template <int NQ>
__device__ __forceinline__ void block_reduce_store_f(float (&v)[NQ], double* out) {
    __shared__ double red[NQ][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        KSum k{v[q], 0.0f};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float s = __shfl_xor_sync(0xffffffffu, k.s, o);
            const float c = __shfl_xor_sync(0xffffffffu, k.c, o);
            k.add(s);
            k.c += c;
        }
        if (lane == 0) red[q][wid] = (double)k.s + (double)k.c;
    }
    __syncthreads();
    if (threadIdx.x < NQ) {
        double s = 0.0;
        for (int w = 0; w < nw; w++) s += red[threadIdx.x][w];
        out[threadIdx.x] = s;
    }
}

__device__ __forceinline__ void set_status(Macro* m, int st) { atomicCAS(&m->status, 0, st); }

// ------------------------------------------------------------------- NR


__device__ __forceinline__ void sinh_cosh(double x, double& sh, double& ch) {
    const double e = exp(x);
    if (x < 700.0) {
        const double ei = 1.0 / e;
        sh = 0.5 * (e - ei);
        ch = 0.5 * (e + ei);
    } else {
        // e^-x is below 1e-304 here: sinh = cosh = e^x / 2 (inf past ~710)
        sh = 0.5 * e;
        ch = sh;
    }
}
// FP32 overflows at x ~ 89 (FP64 at ~710): the argument is capped at 85,
// where the rate is ~1e37 gam_o and any line-search trial is rejected anyway.
__device__ __forceinline__ void sinh_cosh(float x, float& sh, float& ch) {
    const float e = __expf(fminf(x, 85.0f)), ei = __fdividef(1.0f, e);
    sh = 0.5f * (e - ei);
    ch = 0.5f * (e + ei);
}

// StrainRate_Orowan at stress s (constitutive.c:585-725): per slip system the
// resolved shear stress and the sinh glide law with its derivative; returns
// edot (5), the upper triangle of d_edot (15) and the shear rates (shared
// memory column of this thread). bad |= NaN seen (the reference asserts).
// Two passes: the resolved shear stresses of all systems give the mask of
// systems above their passing stress; the glide law then runs over the set
// bits only, lowest first, so a warp iterates max(active per lane) times
// instead of once per system any lane has active. The sums keep the system
// order, so the results are those of one pass over all systems.
// Per-voxel constants of the slip systems staged in shared memory for the
// sweep (column of this thread, stride NR_BLOCK): Schmid vectors at
// [5i+q], tau_pass at [60+i], 1/(tau0+tau_cut) at [72+i], gam_o at [84+i].
constexpr int NSTAGE = 96;

template <typename T>
__device__ __forceinline__ T resolved_shear(const T* cs, const T* s, int i, T (&sc)[5]) {
#pragma unroll
    for (int q = 0; q < 5; q++) sc[q] = cs[(i * 5 + q) * NR_BLOCK];
    return sc[0] * s[0] + sc[1] * s[1] + sc[2] * s[2] + sc[3] * s[3] + sc[4] * s[4];
}

template <typename T>
__device__ __forceinline__ void flow_eval(const NrArgs<T>& a, int nsys, int v, const T* cs,
                                          const T (&s)[6], bool stale, T (&ed)[5], T (&dd)[15], T* gam,
                                          bool& bad, bool want_dd = true) {
    const size_t N = a.g.N;
#pragma unroll
    for (int q = 0; q < 5; q++) ed[q] = (T)0;
#pragma unroll
    for (int q = 0; q < 15; q++) dd[q] = (T)0;
    unsigned act = 0;
    auto pass1 = [&](int i) {
        T sc[5];
        const T rss = resolved_shear<T>(cs, s, i, sc);
        const T tp = stale ? __ldg(a.fc + (size_t)(36 + i) * N + v) : cs[(60 + i) * NR_BLOCK];
        if (fabs(rss) > tp) act |= 1u << i;
        if (gam) gam[i * NR_BLOCK] = (T)0;  // only sweeps that output gamdot keep them
    };
    // FP32: unrolled over the system bound (the loop overhead was a sixth of
    // the pass); FP64 keeps it rolled (its registers are at the limit)
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int i = 0; i < NS; i++) {
            if (i >= nsys) break;
            pass1(i);
        }
    } else {
#pragma unroll 1
        for (int i = 0; i < nsys; i++) pass1(i);
    }
#pragma unroll 1
    while (act) {
        const int i = __ffs(act) - 1;
        act &= act - 1;
        T sc[5];
        const T rss = resolved_shear<T>(cs, s, i, sc);
        const T tp = stale ? __ldg(a.fc + (size_t)(36 + i) * N + v) : cs[(60 + i) * NR_BLOCK];
        const T ar = fabs(rss);
        const T itc = cs[(72 + i) * NR_BLOCK];
        const T go = cs[(84 + i) * NR_BLOCK];
        T sh, ch;
        sinh_cosh((ar - tp) * itc, sh, ch);
        const T g = (rss > (T)0) ? go * sh : -(go * sh);
#pragma unroll
        for (int q = 0; q < 5; q++) ed[q] += sc[q] * g;
        if (want_dd) {
            const T g2 = go * ch * itc;
            int k = 0;
#pragma unroll
            for (int p = 0; p < 5; p++) {
                const T w = sc[p] * g2;
#pragma unroll
                for (int q = p; q < 5; q++) dd[k++] += w * sc[q];
            }
        }
        if (gam) gam[i * NR_BLOCK] = g;
    }
    bool nan = false;
#pragma unroll
    for (int q = 0; q < 5; q++) nan = nan || isnan(ed[q]);
#pragma unroll
    for (int q = 0; q < 15; q++) nan = nan || isnan(dd[q]);
    bad = bad || nan;
}

// FP32 form: the flow rule with the voxel's slip-system constants read from
// the block records in shared memory (two 128-bit reads per system: Schmid
// vector 0..3 | Schmid vector 4, passing stress, 1/(tau0+tau_cut), gamma0_dot).
// rb: this voxel's record of system 0 in float4 units, system i at
// rb + 2 NR_BLOCK i; sw: the voxel's half swap. Same arithmetic as flow_eval.
__device__ __forceinline__ void flow_eval_rec(const NrArgs<float>& a, int nsys, int v, const float4* rb, int sw,
                                              const float (&s)[6], bool stale, float (&ed)[5], float (&dd)[15],
                                              bool& bad) {
    const size_t N = a.g.N;
#pragma unroll
    for (int q = 0; q < 5; q++) ed[q] = 0.f;
#pragma unroll
    for (int q = 0; q < 15; q++) dd[q] = 0.f;
    unsigned act = 0;
#pragma unroll
    for (int i = 0; i < NS; i++) {
        if (i >= nsys) break;
        const float4 h0 = rb[2 * NR_BLOCK * i + sw], h1 = rb[2 * NR_BLOCK * i + (sw ^ 1)];
        const float rss = h0.x * s[0] + h0.y * s[1] + h0.z * s[2] + h0.w * s[3] + h1.x * s[4];
        const float tp = stale ? __ldg(a.fc + (size_t)(36 + i) * N + v) : h1.y;
        if (fabsf(rss) > tp) act |= 1u << i;
    }
#pragma unroll 1
    while (act) {
        const int i = __ffs(act) - 1;
        act &= act - 1;
        const float4 h0 = rb[2 * NR_BLOCK * i + sw], h1 = rb[2 * NR_BLOCK * i + (sw ^ 1)];
        const float sc[5] = {h0.x, h0.y, h0.z, h0.w, h1.x};
        const float rss = sc[0] * s[0] + sc[1] * s[1] + sc[2] * s[2] + sc[3] * s[3] + sc[4] * s[4];
        const float tp = stale ? __ldg(a.fc + (size_t)(36 + i) * N + v) : h1.y;
        const float ar = fabsf(rss);
        const float itc = h1.z;
        const float go = h1.w;
        float sh, ch;
        sinh_cosh((ar - tp) * itc, sh, ch);
        const float g = (rss > 0.f) ? go * sh : -(go * sh);
        const float g2 = go * ch * itc;
#pragma unroll
        for (int q = 0; q < 5; q++) ed[q] += sc[q] * g;
        int k = 0;
#pragma unroll
        for (int p = 0; p < 5; p++) {
            const float w = sc[p] * g2;
#pragma unroll
            for (int q = p; q < 5; q++) dd[k++] += w * sc[q];
        }
    }
    bool nan = false;
#pragma unroll
    for (int q = 0; q < 5; q++) nan = nan || isnan(ed[q]);
#pragma unroll
    for (int q = 0; q < 15; q++) nan = nan || isnan(dd[q]);
    bad = bad || nan;
}

// FP32 Jacobian of the flow rule, d_edot/d_sigma (upper triangle of the 5x5
// deviatoric block), at stress s from the voxel's FP32 constant records in
// global memory (the FP64 refinement's correction matrix).
__device__ __forceinline__ void jac_rec32(const float* nrc, int v, int nsys, const float (&s)[6], float (&dd)[15]) {
#pragma unroll
    for (int q = 0; q < 15; q++) dd[q] = 0.f;
#pragma unroll 1
    for (int i = 0; i < nsys; i++) {
        const float4 h0 = __ldg(reinterpret_cast<const float4*>(nrc + nrc_index(v, i, 0)));
        const float4 h1 = __ldg(reinterpret_cast<const float4*>(nrc + nrc_index(v, i, 1)));
        const float sc[5] = {h0.x, h0.y, h0.z, h0.w, h1.x};
        const float rss = sc[0] * s[0] + sc[1] * s[1] + sc[2] * s[2] + sc[3] * s[3] + sc[4] * s[4];
        if (!(fabsf(rss) > h1.y)) continue;
        float sh, ch;
        sinh_cosh((fabsf(rss) - h1.y) * h1.z, sh, ch);
        const float g2 = h1.w * ch * h1.z;
        int k = 0;
#pragma unroll
        for (int p = 0; p < 5; p++) {
            const float w = sc[p] * g2;
#pragma unroll
            for (int q = p; q < 5; q++) dd[k++] += w * sc[q];
        }
    }
}

// Bulk copies global -> shared memory completing on an mbarrier (one phase).
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for phase 0 of the barrier a bounded number of times (each try may
// suspend the thread for a short, system-dependent time); false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar) {
    for (int k = 0; k < (1 << 18); k++)
        if (mbar_try_wait(bar, 0)) return true;
    return false;
}

// Quotient in the working precision: IEEE division in FP64 (parity with the
// reference), the fast reciprocal-based quotient in FP32 (within 2 ulp; the
// FP32 form's tolerance is set by its own NR tolerance, far above that).
__device__ __forceinline__ double fdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }

// Packed symmetric 6x6: index of (i,j), i <= j.
__host__ __device__ constexpr int sidx(int i, int j) { return i * 6 - i * (i - 1) / 2 + (j - i); }

// Solve M x = b for symmetric positive definite M (packed upper, 21 entries)
// by LDL^T without pivoting. Returns false when a pivot is not positive.
// Every loop has a constant trip count with the triangle as a guard, so the
// loops unroll whole and m stays in registers (triangular bounds left the
// packed matrix in local memory).
template <typename T>
__device__ __forceinline__ bool ldl_factor(T (&m)[21], T (&id)[6]) {
    // in place: m[sidx(k,i)] holds L(i,k) for i > k and d_k on the diagonal
    bool ok = true;
#pragma unroll
    for (int j = 0; j < 6; j++) {
        T dj = m[sidx(j, j)];
#pragma unroll
        for (int k = 0; k < 6; k++)
            if (k < j) dj -= m[sidx(k, j)] * m[sidx(k, j)] * m[sidx(k, k)];
        m[sidx(j, j)] = dj;
        ok = ok && (dj > (T)0);
        id[j] = fdiv((T)1, dj);
#pragma unroll
        for (int i = 0; i < 6; i++) {
            if (i > j) {
                T t = m[sidx(j, i)];
#pragma unroll
                for (int k = 0; k < 6; k++)
                    if (k < j) t -= m[sidx(k, i)] * m[sidx(k, j)] * m[sidx(k, k)];
                m[sidx(j, i)] = t * id[j];
            }
        }
    }
    return ok;
}

template <typename T>
__device__ __forceinline__ void ldl_subst(const T (&m)[21], const T (&id)[6], const T (&b)[6], T (&x)[6]) {
    T y[6];
#pragma unroll
    for (int i = 0; i < 6; i++) {
        T t = b[i];
#pragma unroll
        for (int k = 0; k < 6; k++)
            if (k < i) t -= m[sidx(k, i)] * y[k];
        y[i] = t;
    }
#pragma unroll
    for (int i = 5; i >= 0; i--) {
        T t = y[i] * id[i];
#pragma unroll
        for (int k = 0; k < 6; k++)
            if (k > i) t -= m[sidx(i, k)] * x[k];
        x[i] = t;
    }
}

template <typename T>
__device__ __forceinline__ bool ldl_solve(T (&m)[21], const T (&b)[6], T (&x)[6]) {
    T id[6];
    const bool ok = ldl_factor<T>(m, id);
    ldl_subst<T>(m, id, b, x);
    return ok;
}

template <typename T>
__device__ __forceinline__ void mat6v(const T (&m)[6][6], const T* x, T* y) {
#pragma unroll
    for (int i = 0; i < 6; i++) {
        T s = (T)0;
#pragma unroll
        for (int j = 0; j < 6; j++) s += m[i][j] * x[j];
        y[i] = s;
    }
}

// S x with S read from the per-orientation table (L1-resident: voxels of a
// grain share it). FP64 rows hold S_gr (36) and the packed NR matrix base
// S066 + sym(S_gr) (21); FP32 rows hold the packed sym(S_gr) alone (21), which
// serves both (36 + 21 loads per Newton step become 21).
// The 21 packed values of an FP32 orientation row (rows are 256-byte aligned):
// five 128-bit loads and one scalar load.
__device__ __forceinline__ void load_sym21(const float* sg, float (&u)[21]) {
    const float4* s4 = reinterpret_cast<const float4*>(sg);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const float4 t = __ldg(s4 + k);
        u[4 * k] = t.x;
        u[4 * k + 1] = t.y;
        u[4 * k + 2] = t.z;
        u[4 * k + 3] = t.w;
    }
    u[20] = __ldg(sg + 20);
}

template <typename T>
__device__ __forceinline__ void sgr_v(const T* sg, const T* x, T* y) {
    if constexpr (sizeof(T) == 4) {
        T u[21];
        load_sym21(sg, u);
#pragma unroll
        for (int i = 0; i < 6; i++) {
            T s = (T)0;
#pragma unroll
            for (int j = 0; j < 6; j++) s += u[i <= j ? sidx(i, j) : sidx(j, i)] * x[j];
            y[i] = s;
        }
    } else {
#pragma unroll
        for (int i = 0; i < 6; i++) {
            T s = (T)0;
#pragma unroll
            for (int j = 0; j < 6; j++) s += __ldg(sg + i * 6 + j) * x[j];
            y[i] = s;
        }
    }
}

// Packed base of the NR matrix, S066 + sym(S_gr), of the voxel's orientation.
template <typename T>
__device__ __forceinline__ void nr_matrix_base(const T* sg, const T (&S66)[6][6], T (&m)[21]) {
    if constexpr (sizeof(T) == 4) {
        T u[21];
        load_sym21(sg, u);
#pragma unroll
        for (int i = 0; i < 6; i++)
#pragma unroll
            for (int j = 0; j < 6; j++)
                if (j >= i) m[sidx(i, j)] = S66[i][j] + u[sidx(i, j)];
    } else {
#pragma unroll
        for (int k = 0; k < 21; k++) m[k] = __ldg(sg + 36 + k);
    }
}

// Warp-level partial sums without a block barrier: every warp writes its own
// row of NPART_NR values (FP64 sweeps: doubles; FP32 sweeps: compensated
// within the warp, stored as the float pair sum + compensation). The 15
// values (padded to 16) are reduced by recursive halving: at each of the
// first four levels a lane keeps half of its values and receives the
// partner's copy of that half, so the warp exchanges 8+4+2+1 values, then
// the last level sums lane pairs; lane 2k ends with value k. 16 shuffle
// steps instead of 15 butterflies of 5.
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ void warp_store(double (&q)[NPART_NR], double* row) {
    const int lane = threadIdx.x & 31;
    double v[16];
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = k < NPART_NR ? q[k] : 0.0;
#pragma unroll
    for (int st = 0; st < 4; st++) {
        const int h = 8 >> st, o = 16 >> st;
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < h; j++) {
            const double send = up ? v[j] : v[j + h];
            const double keep = up ? v[j + h] : v[j];
            v[j] = keep + __shfl_xor_sync(kFull, send, o);
        }
    }
    v[0] += __shfl_xor_sync(kFull, v[0], 1);
    if (!(lane & 1) && (lane >> 1) < NPART_NR) row[lane >> 1] = v[0];
}
__device__ __forceinline__ void warp_store(float (&q)[NPART_NR], double* row) {
    const int lane = threadIdx.x & 31;
    float s[16], c[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        s[k] = k < NPART_NR ? q[k] : 0.0f;
        c[k] = 0.0f;
    }
#pragma unroll
    for (int st = 0; st < 5; st++) {
        const int h = st < 4 ? 8 >> st : 1, o = 16 >> st;
        const bool up = st < 4 && (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < h; j++) {
            const float ss = up ? s[j] : s[j + (st < 4 ? h : 0)];
            const float cs = up ? c[j] : c[j + (st < 4 ? h : 0)];
            KSum ks{up ? s[j + h] : s[j], up ? c[j + h] : c[j]};
            const float rs = __shfl_xor_sync(kFull, ss, o);
            const float rc = __shfl_xor_sync(kFull, cs, o);
            ks.add(rs);
            ks.c += rc;
            s[j] = ks.s;
            c[j] = ks.c;
        }
    }
    if (!(lane & 1) && (lane >> 1) < NPART_NR)
        reinterpret_cast<float2*>(row)[lane >> 1] = make_float2(s[0], c[0]);
}

// Asynchronous copy of one scalar from global to this thread's shared-memory
// column (no register round trip, all copies of a thread in flight at once).
template <typename T>
__device__ __forceinline__ void stage_async(T* dst, const T* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(src), "n"(sizeof(T)) : "memory");
}
__device__ __forceinline__ void stage_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// FP32 loop sweep: a Newton step no longer than 30 tolerances of |lambda|
// (3e-4 at the default 1e-5) ends the NR; squared ratio
constexpr float NR32_ACCEPT2 = 900.0f;

// Resident NR blocks of two warps per SM the register budget is set for.
// FP32: 9, as many as the 24 KB of constant records per block allow in
// shared memory (18 warps per SM): the sweep then fits 96 registers without
// spills, where an open budget took 123 and left 16 warps per SM (0.260 ->
// 0.242 ms at 128^3). FP64: 4 (228 registers, 55 KB of staging per block).
template <typename T> struct NrMinBlocks { static constexpr int v = 4; };
template <> struct NrMinBlocks<float> { static constexpr int v = 9; };

// One UpdateStress sweep (evolution.c:181-423). The line search of the
// NR_MODIFIED build runs as a small state machine so the flow rule has a
// single call site: a MAIN step evaluates the flow rule at sigma, solves for
// the Newton step and either applies it (plain) or proposes the first trial
// point; a TRIAL step evaluates the flow rule there and accepts the point,
// backtracks or gives up (evolution.c:337-370). An accepted trial's
// evaluation is the next MAIN's evaluation.
// B: batched launch (C066/S066 staged in shared memory at sS/sC); otherwise
// they are read from the kernel's constant bank.
template <typename T, int LS, bool B>
__device__ __forceinline__ void nr_body(const NrArgs<T>& a, int bid, unsigned char* nr_smem,
                                        const T* sS, const T* sC) {
    T* s_stage = reinterpret_cast<T*>(nr_smem);
    const T(&S66)[6][6] = B ? *reinterpret_cast<const T(*)[6][6]>(sS) : a.mat.s066;
    const T(&C66)[6][6] = B ? *reinterpret_cast<const T(*)[6][6]>(sC) : a.mat.c066;
    const int v = bid * NR_BLOCK + threadIdx.x;
    const int N = a.g.N;
    const T dt = a.mat.dt;
    T* stg = s_stage + threadIdx.x;
    T* gam = sizeof(T) == 8 ? s_stage + NSTAGE * NR_BLOCK + threadIdx.x : nullptr;
    T pe = 0, ps = 0, ss[6] = {0, 0, 0, 0, 0, 0}, s1[6] = {0, 0, 0, 0, 0, 0};
    int nr = 0;
    bool bad = false, sing = false, lsfail = false, tmo = false, waited = false;
    // FP32 sweeps: the block's constant records (24 KB) arrive by bulk copies
    // issued by one thread, overlapping the state loads of every thread
    unsigned long long* cbar = nullptr;
    if constexpr (sizeof(T) == 4) {
        cbar = reinterpret_cast<unsigned long long*>(nr_smem + (size_t)NRC_BLOCK_FLOATS * sizeof(float));
        if (threadIdx.x == 0) mbar_init(cbar, 1);
        __syncthreads();
        if (threadIdx.x == 0) {
            constexpr unsigned SYS_BYTES = NR_BLOCK * NRC_REC * sizeof(float);
            mbar_expect_tx(cbar, NS * SYS_BYTES);
            const float* src = a.nrc + (size_t)bid * NRC_BLOCK_FLOATS;
#pragma unroll 1
            for (int i = 0; i < NS; i++)
                bulk_g2s(nr_smem + (size_t)i * SYS_BYTES, src + (size_t)i * NR_BLOCK * NRC_REC, SYS_BYTES, cbar);
        }
    }
    const bool stale0 = a.stale_mode && a.macro->iter == 0;
    const int ph = (v < N) ? a.phase[v] : 1;
    const PhaseK<T>& P = a.mat.ph[ph - 1];
    if (v < N && !P.crystal) {
#pragma unroll
        for (int c = 0; c < 6; c++) a.sig[(size_t)c * N + v] = (T)0;
        if (a.edot)
#pragma unroll
            for (int c = 0; c < 5; c++) a.edot[(size_t)c * N + v] = (T)0;
    } else if (v < N) {
        int nsys = P.n_sys;
        const T* sg = a.sgr + (size_t)a.orient[v] * SGR_STRIDE;
        if constexpr (sizeof(T) == 8) {
            // the staging copies overlap the loads of the voxel's state below
            for (int i = 0; i < nsys; i++) {
#pragma unroll
                for (int q = 0; q < 5; q++)
                    stage_async<T>(stg + (i * 5 + q) * NR_BLOCK, a.schm + (size_t)(i * 5 + q) * N + v);
#pragma unroll
                for (int q = 0; q < 3; q++)
                    stage_async<T>(stg + (60 + 12 * q + i) * NR_BLOCK, a.fc + (size_t)(12 * q + i) * N + v);
            }
            stage_commit();
        }
        T lam[6], sig[6], av[6], old[6], step[6], te[6];
#pragma unroll
        for (int c = 0; c < 6; c++) {
            lam[c] = a.sig[(size_t)c * N + v];
            sig[c] = lam[c];
            av[c] = a.epsb[(size_t)c * N + v] - a.dg[(size_t)c * N + v];
        }
        if constexpr (sizeof(T) == 8) {
            stage_wait();
        } else {
            // a copy that never completes stops the RVE with a timeout status;
            // the voxel then runs without slip systems (its result is unused)
            waited = true;
            if (!mbar_wait_bounded(cbar)) {
                tmo = true;
                nsys = 0;
            }
        }
        T signorm = 0;
#pragma unroll
        for (int c = 0; c < 6; c++) signorm += lam[c] * lam[c];
        signorm = sqrt(signorm);
        T ed[5], dd[15], edot_out[5] = {0, 0, 0, 0, 0};
        // NR convergence: |sig - old| / |lambda| <= tol (evolution.c:386-391); the
        // FP32 form compares the squared step with (tol |lambda|)^2 instead
        T erral, tolc;
        if constexpr (sizeof(T) == 4) {
            tolc = (a.tol * signorm) * (a.tol * signorm);
            erral = (T)100 * tolc + (T)1e-30;
        } else {
            tolc = fabs(a.tol);
            erral = (T)10 * a.tol;
        }
        T ce = 0, cs = 0;
        T f_old = 0, slope = 0, alam = 1, alam2 = 0, alamin = 0;
        bool trial = false, accepted = false;
        int it = 0, guard = 0;
        // end of a Newton or line-search step: the NR convergence measure
        // (evolution.c:386-391); the voxel's error terms of its last step are
        // formed after the loop
        auto finish_step = [&]() {
            T cnr = 0;
#pragma unroll
            for (int c = 0; c < 6; c++) cnr += (sig[c] - old[c]) * (sig[c] - old[c]);
            if constexpr (sizeof(T) == 4) erral = cnr;  // squared step, against tolc
            else erral = fdiv(sqrt(cnr), signorm);
        };
        // FP64 refinement of the FP32-bulk form (mixed): from the converged FP32
        // stress, corrections with an FP32 Jacobian and LDL^T (from the FP32
        // constant records) applied to FP64 residuals with FP64 flow-rule rates,
        // until the step meets the FP64 NR tolerance. The Jacobian is rebuilt at
        // the current stress when a step does not shrink; a voxel still not
        // converged after MIX_ITMAX corrections goes through the FP64 line-search
        // NR below from where it stands. The rates and slip rates kept are those
        // of the evaluation before the last step, as in the line-search loop.
        bool mixed_done = false;
        if constexpr (sizeof(T) == 8) {
            if (a.mixed) {
                constexpr int MIX_ITMAX = 8;
                float mf[21], idf[6];
                bool need_jac = true;
                T prev = (T)0;
                for (int k = 0; k < MIX_ITMAX && !mixed_done; k++) {
                    T ed[5], dd[15];
                    flow_eval<T>(a, nsys, v, stg, sig, false, ed, dd, a.gamdot ? gam : nullptr, bad, false);
                    if (bad) break;
#pragma unroll
                    for (int q = 0; q < 5; q++) edot_out[q] = ed[q];
                    T Ss[6], dl[6], rhs[6];
                    sgr_v<T>(sg, sig, Ss);
#pragma unroll
                    for (int c = 0; c < 6; c++) {
                        te[c] = av[c] + (c < 5 ? ed[c] * dt : (T)0) + Ss[c];
                        dl[c] = sig[c] - lam[c];
                    }
                    mat6v<T>(S66, dl, rhs);
                    if (need_jac) {
                        float s32[6], dd32[15];
#pragma unroll
                        for (int c = 0; c < 6; c++) s32[c] = (float)sig[c];
                        jac_rec32(a.nrc, v, nsys, s32, dd32);
                        const float dtf = (float)dt;
#pragma unroll
                        for (int q = 0; q < 21; q++) mf[q] = (float)__ldg(sg + 36 + q);
                        {
                            int q = 0;
#pragma unroll
                            for (int p = 0; p < 5; p++)
#pragma unroll
                                for (int r = p; r < 5; r++) mf[sidx(p, r)] += dtf * dd32[q++];
                        }
                        if (!ldl_factor<float>(mf, idf)) { sing = true; break; }
                        need_jac = false;
                    }
                    float r32[6], x32[6];
#pragma unroll
                    for (int c = 0; c < 6; c++) r32[c] = (float)(rhs[c] + te[c]);
                    ldl_subst<float>(mf, idf, r32, x32);
                    T cnr = 0;
#pragma unroll
                    for (int c = 0; c < 6; c++) {
                        old[c] = sig[c];
                        sig[c] -= (T)x32[c];
                        const T d = sig[c] - old[c];
                        cnr += d * d;
                    }
                    it++;
                    const T st = sqrt(cnr);
                    if (st <= a.tol * signorm) mixed_done = true;
                    else if (k > 0 && st > (T)0.5 * prev) need_jac = true;
                    prev = st;
                }
            }
        }
        // One flow-rule evaluation per pass. A pass at a line-search trial
        // point evaluates its merit; when the point is accepted, the Newton step
        // that starts there runs in the same pass with that evaluation (the
        // reference's next iteration reuses it too), so lanes of a warp that
        // accept trial points stay with lanes that take plain Newton steps.
        if (!mixed_done) for (;;) {
            if (!trial) {
                if (!(it < a.itmax && fabs(erral) > tolc)) break;
                it++;
#pragma unroll
                for (int c = 0; c < 6; c++) old[c] = sig[c];
            }
            if constexpr (sizeof(T) == 4)
                flow_eval_rec(a, nsys, v, reinterpret_cast<const float4*>(nr_smem) + 2 * threadIdx.x,
                              (threadIdx.x >> 2) & 1, sig, !trial && stale0 && it == 1, ed, dd, bad);
            else
                flow_eval<T>(a, nsys, v, stg, sig, !trial && stale0 && it == 1, ed, dd, a.gamdot ? gam : nullptr,
                             bad);
            if (bad) break;
            if (trial) {
                // TRIAL: merit at sig = old + alam step (NR_quality, evolution.c:115-154)
                T Ss[6], tt6[6], Rt[6], fnew = 0;
                sgr_v<T>(sg, sig, Ss);
#pragma unroll
                for (int c = 0; c < 6; c++) tt6[c] = av[c] + (c < 5 ? ed[c] * dt : (T)0) + Ss[c];
                mat6v<T>(C66, tt6, Rt);
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    const T r = sig[c] - lam[c] + Rt[c];
                    fnew += r * r;
                }
                fnew *= (T)0.5;
                if (alam < alamin) {
                    // no acceptable point: back to the base point, which the next
                    // pass evaluates again (evolution.c:345-349)
#pragma unroll
                    for (int c = 0; c < 6; c++) sig[c] = old[c];
                    trial = false;
                    finish_step();
                    continue;
                }
                if (!(fnew <= f_old + (T)1e-4 * alam * slope)) {
                    T tmplam;
                    if (fabs(alam - (T)1) < (T)1e-4) {
                        tmplam = -slope / ((T)2 * (fnew - f_old - slope));
                    } else {
                        const T f2 = 0;  // never updated in the reference
                        const T rhs1 = fnew - f_old - alam * slope;
                        const T rhs2 = f2 - f_old - alam2 * slope;
                        const T ac = (rhs1 / (alam * alam) - rhs2 / (alam2 * alam2)) / (alam - alam2);
                        const T bc = (-alam2 * rhs1 / (alam * alam) + alam * rhs2 / (alam2 * alam2)) /
                                     (alam - alam2);
                        if (fabs(ac) < (T)1e-4) {
                            tmplam = -slope / ((T)2 * bc);
                        } else {
                            const T disc = bc * bc - (T)3 * ac * slope;
                            if (disc < (T)0) tmplam = (T)0.5 * alam;
                            else if (bc <= (T)0) tmplam = (-bc + sqrt(disc)) / ((T)3 * ac);
                            else tmplam = -slope / (bc + sqrt(disc));
                        }
                        if (tmplam > (T)0.5 * alam) tmplam = (T)0.5 * alam;
                    }
                    alam2 = alam;
                    alam = fmax(tmplam, (T)0.1 * alam);
#pragma unroll
                    for (int c = 0; c < 6; c++) sig[c] = old[c] + alam * step[c];
                    if (++guard > 200) { lsfail = true; break; }
                    continue;
                }
                // accepted: the Newton step from this point uses this evaluation
                trial = false;
                finish_step();
                if (!(it < a.itmax && fabs(erral) > tolc)) break;
                it++;
#pragma unroll
                for (int c = 0; c < 6; c++) old[c] = sig[c];
            }
            // MAIN: Newton step at sig
            bool finish = false;
#pragma unroll
            for (int q = 0; q < 5; q++) edot_out[q] = ed[q];
            // te = tot_eps - strain = (Eps - strain) + edot dt + S sig
            {
                T Ss[6];
                sgr_v<T>(sg, sig, Ss);
#pragma unroll
                for (int c = 0; c < 6; c++) te[c] = av[c] + (c < 5 ? ed[c] * dt : (T)0) + Ss[c];
            }
            // M = S066 + sym(S) + dt d_edot (the first two per orientation);
            // rhs = S066 R = S066 (sig - lam) + te
            T m[21];
            nr_matrix_base<T>(sg, S66, m);
            {
                int k = 0;
#pragma unroll
                for (int p = 0; p < 5; p++)
#pragma unroll
                    for (int q = p; q < 5; q++) m[sidx(p, q)] += dt * dd[k++];
            }
            T dl[6], rhs[6];
#pragma unroll
            for (int c = 0; c < 6; c++) dl[c] = sig[c] - lam[c];
            mat6v<T>(S66, dl, rhs);
#pragma unroll
            for (int c = 0; c < 6; c++) rhs[c] += te[c];
            if (!ldl_solve<T>(m, rhs, step)) { sing = true; break; }
            if (!LS) {
#pragma unroll
                for (int c = 0; c < 6; c++) sig[c] -= step[c];
                finish = true;
            } else {
                // NR_MODIFIED (evolution.c:284-336). slope = (J^T R).step with
                // step = -J^-1 R capped at length 10, i.e. -|R|^2 times the cap
                // factor; used directly because through an ill-conditioned J
                // the rounded product can change sign.
                T nrm = 0;
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    step[c] = -step[c];
                    nrm += step[c] * step[c];
                }
                nrm = sqrt(nrm);
                bool whole = false;
                if (a.quick_accept && nrm <= (T)10) {
                    // a step below the NR tolerance ends the NR whatever the line
                    // search would pick (a shorter step only lowers erral): take it
                    // whole; the trial's merit would decide a change below the
                    // tolerance. FP32-bulk form only. A NaN step fails the test and
                    // takes the line search's error path.
                    T cnr = 0;
#pragma unroll
                    for (int c = 0; c < 6; c++) {
                        const T d = (old[c] + step[c]) - old[c];
                        cnr += d * d;
                    }
                    if (sizeof(T) == 4 ? cnr <= tolc : fdiv(sqrt(cnr), signorm) <= a.tol) {
#pragma unroll
                        for (int c = 0; c < 6; c++) sig[c] = old[c] + step[c];
                        whole = true;
                        finish = true;
                    } else if (sizeof(T) == 4 && cnr <= NR32_ACCEPT2 * tolc) {
                        // FP32 loop: a Newton step of relative length s <= 30 tol
                        // (3e-4) leaves an error ~K s^2 (quadratic convergence), below
                        // the tolerance for K up to ~100; the step that would confirm
                        // it is, in FP32 at that distance, dominated by the rounding of
                        // the residual's large terms. Take the step and end the NR.
#pragma unroll
                        for (int c = 0; c < 6; c++) sig[c] = old[c] + step[c];
                        whole = true;
                        finish = true;
                        accepted = true;
                    }
                }
                if (!whole) {
                    T CR[6];
                    mat6v<T>(C66, te, CR);
                    f_old = 0;
#pragma unroll
                    for (int c = 0; c < 6; c++) {
                        const T r = dl[c] + CR[c];
                        f_old += r * r;
                    }
                    slope = -f_old;
                    f_old *= (T)0.5;
                    if (nrm > (T)10) {
                        const T cap = fdiv((T)10, nrm);
#pragma unroll
                        for (int c = 0; c < 6; c++) step[c] *= cap;
                        slope *= cap;
                    }
                }
                if (whole) {
                } else if (!(slope < (T)0)) {
                    if (slope != (T)0) { lsfail = true; break; }
                    finish = true;  // R == 0: at the root already
                } else {
                    T test = 0;
#pragma unroll
                    for (int c = 0; c < 6; c++) {
                        const T tt = fdiv(fabs(step[c]), fmax(fabs(old[c]), (T)1));
                        if (tt > test) test = tt;
                    }
                    alamin = fdiv((T)1e-7, test);
                    alam = 1;
                    alam2 = 0;
#pragma unroll
                    for (int c = 0; c < 6; c++) sig[c] = old[c] + step[c];
                    trial = true;
                    guard = 0;
                }
            }
            if (finish) finish_step();
            if (accepted) erral = (T)0;
        }
        // the voxel's error terms at the end of its last step
        {
#pragma unroll
            for (int c = 0; c < 6; c++) {
                ce += te[c] * te[c];
                cs += (sig[c] - lam[c]) * (sig[c] - lam[c]);
            }
            if constexpr (sizeof(T) == 4) {
                // FP32 form: at the NR solution tot_eps - eps = -S066 (sig - lambda);
                // evaluated at the final stress it carries no lag of the last
                // Newton step (the reference takes tot_eps before that step, which
                // at the FP32 NR tolerance would floor Err_e near 1e-5).
                T d6[6], q6[6];
#pragma unroll
                for (int c = 0; c < 6; c++) d6[c] = sig[c] - lam[c];
                mat6v<T>(S66, d6, q6);
                ce = 0;
#pragma unroll
                for (int c = 0; c < 6; c++) ce += q6[c] * q6[c];
            }
            ce = sqrt(ce);
            cs = sqrt(cs);
        }
        nr = it;
#pragma unroll
        for (int c = 0; c < 6; c++) a.sig[(size_t)c * N + v] = sig[c];
        if (a.edot)
#pragma unroll
            for (int c = 0; c < 5; c++) a.edot[(size_t)c * N + v] = edot_out[c];
        if (a.gamdot)
            for (int i = 0; i < nsys; i++) a.gamdot[(size_t)i * N + v] = gam[i * NR_BLOCK];
        pe = ce;
        ps = cs;
#pragma unroll
        for (int c = 0; c < 6; c++) {
            ss[c] = sig[c];
            s1[c] = (ph == 1) ? sig[c] : (T)0;
        }
    }
    if constexpr (sizeof(T) == 4) {
        // every thread has seen the copies complete (or given up) before the
        // block's shared memory is released
        if (!waited && !mbar_wait_bounded(cbar)) tmo = true;
        if (tmo) {
            mbar_wait_bounded(cbar);
            set_status(a.macro, 10);
        }
    }
    if (bad) set_status(a.macro, 4);
    if (sing) set_status(a.macro, 5);
    if (lsfail) set_status(a.macro, 6);
    T q[NPART_NR];
    q[0] = pe;
    q[1] = ps;
#pragma unroll
    for (int c = 0; c < 6; c++) {
        q[2 + c] = ss[c];
        q[8 + c] = s1[c];
    }
    q[14] = (T)nr;
    const int warp = (bid * NR_BLOCK + threadIdx.x) >> 5;
    warp_store(q, a.part + (size_t)warp * NPART_NR);
}

template <typename T> __device__ __forceinline__ constexpr size_t nr_smem_main() {
    return sizeof(T) == 4 ? (size_t)NRC_BLOCK_FLOATS * sizeof(float) + 16
                          : (size_t)(NSTAGE + NS) * NR_BLOCK * sizeof(T);
}

template <typename T, int LS>
__global__ void __launch_bounds__(NR_BLOCK, NrMinBlocks<T>::v) k_nr(const __grid_constant__ NrArgs<T> a) {
    extern __shared__ __align__(16) unsigned char nr_smem[];
    if (!gate_open(a.macro, a.gate)) return;
    nr_body<T, LS, false>(a, blockIdx.x, nr_smem, nullptr, nullptr);
}

template <typename T, int LS>
__global__ void __launch_bounds__(NR_BLOCK, NrMinBlocks<T>::v) kb_nr(const NrArgs<T>* __restrict__ tab,
                                                                     const int2* __restrict__ map) {
    extern __shared__ __align__(16) unsigned char nr_smem[];
    const int2 m = map[blockIdx.x];
    const NrArgs<T>& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    T* sm = reinterpret_cast<T*>(nr_smem + nr_smem_main<T>());
    for (int i = threadIdx.x; i < 36; i += NR_BLOCK) {
        sm[i] = (&a.mat.s066[0][0])[i];
        sm[36 + i] = (&a.mat.c066[0][0])[i];
    }
    __syncthreads();
    nr_body<T, LS, true>(a, m.y, nr_smem, sm, sm + 36);
}

// ---------------------------------------------------------------- macro


// get_smacro and the loop test (evolution.c:590-664, 1227-1252, 1150) on the
// FP64 totals; thread 0 of the last block. Everything is computed in
// registers and written to the macro state once at the end (the state lives
// in global memory, where every read after a write would wait on L2).
__device__ void macro_update(const LoopCfg& c, Macro* m, const double* tot) {
    double s6[6], s16[6], sa[3][3], s1a[3][3], dE[3][3];
    for (int q = 0; q < 6; q++) {
        s6[q] = tot[2 + q];
        s16[q] = tot[8 + q];
    }
    b6_to_sym<double>(s6, sa);
    b6_to_sym<double>(s16, s1a);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            sa[i][j] = sa[i][j] * c.wgt;
            s1a[i][j] = s1a[i][j] * (c.wgt / c.wgt_ph1);
            dE[i][j] = 0.0;
        }
    const int IJV[2][6] = {{0, 1, 2, 1, 0, 0}, {0, 1, 2, 2, 2, 1}};
    for (int i = 0; i < 6; i++) {
        const int ii = IJV[0][i], jj = IJV[1][i];
        double d = 0.0;
        if (c.vflag[i] == 0)
            for (int k = 0; k < 6; k++) {
                const int kk = IJV[0][k], ll = IJV[1][k];
                d += c.s0[ii][jj][kk][ll] * c.sflag[k] * (c.scauchy[kk][ll] - sa[kk][ll]);
            }
        dE[ii][jj] = d;
    }
    double dE9[9];
    {
        double e6[6];
        sym_to_b6<double>(dE, e6);
        for (int q = 0; q < 6; q++) dE9[q] = e6[q];
        dE9[6] = 0.5 * (dE[0][1] - dE[1][0]);
        dE9[7] = 0.5 * (dE[0][2] - dE[2][0]);
        dE9[8] = 0.5 * (dE[1][2] - dE[2][1]);
    }
    // s_vm: the reference's trace term reads SigDevAvg[3][3], one element past
    // the array; in its global layout that is SigAvg1[0][0].
    double s_vm, s_vm1;
    {
        double v6[6], dev[3][3];
        sym_to_b6<double>(sa, v6);
        v6[5] = 0.0;
        b6_to_sym<double>(v6, dev);
        const double oob = s1a[0][0];
        double s = 0.0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                if (i != j) s += dev[i][j] * dev[i][j];
                else {
                    const double d = dev[i][j] - (dev[1][1] + dev[2][2] + oob) / 3.0;
                    s += d * d;
                }
            }
        s_vm = sqrt(1.5 * s);
        sym_to_b6<double>(s1a, v6);
        v6[5] = 0.0;
        b6_to_sym<double>(v6, dev);
        s = 0.0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) s += dev[i][j] * dev[i][j];
        s_vm1 = sqrt(1.5 * s);
    }
    const double e_vm = m->e_vm;
    double ee = tot[0] * c.wgt, es = tot[1] * c.wgt;
    if (fabs(e_vm) < 1E-5) ee = 0.0;
    else ee /= e_vm;
    es /= s_vm;
    const int iter = m->iter + 1;
    const double mx = (fabs(es) > fabs(ee)) ? fabs(es) : fabs(ee);
    const int converged = !(mx > c.err_tol);
    const int status = m->status;
    const long long nr = m->nr_iters;
    double acum[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) acum[i][j] = m->dE_acum[i][j] + dE[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            m->sig_avg[i][j] = sa[i][j];
            m->sig_avg1[i][j] = s1a[i][j];
            m->dE[i][j] = dE[i][j];
            m->dE_acum[i][j] = acum[i][j];
        }
    for (int q = 0; q < 9; q++) m->dE9[q] = dE9[q];
    m->s_vm = s_vm;
    m->s_vm1 = s_vm1;
    m->err_e_sum = tot[0];
    m->err_s_sum = tot[1];
    m->err_e = ee;
    m->err_s = es;
    m->nr_iters = nr + (long long)tot[14];
    m->iter = iter;
    m->converged = converged;
    m->done = converged || iter >= c.iter_max || status != 0;
}

// Deterministic two-level sum of the NR warp partials: each block sums a
// contiguous range of rows in a fixed order; the last block to finish sums
// the block rows in order and runs the macro update.
// bid: block index within the RVE's MACRO_BLOCKS blocks.
// Accumulators of the macro sums: FP64 for the FP64 sweep's rows; for the
// FP32 sweep's rows, float pairs (hi, lo) added exactly as a double-float
// (two-sum of the high parts, then the low parts), which keeps ~44 bits on
// the FP32 pipe instead of the narrow FP64 one.
struct AccD {
    double v;
    __device__ __forceinline__ static AccD zero() { return {0.0}; }
    __device__ __forceinline__ static AccD load(const double* p) { return {*p}; }
    __device__ __forceinline__ static AccD load_cg(const double* p) { return {__ldcg(p)}; }
    __device__ __forceinline__ void add(const AccD& b) { v += b.v; }
    __device__ __forceinline__ AccD shfl(int o) const { return {__shfl_xor_sync(0xffffffffu, v, o)}; }
    __device__ __forceinline__ void store(double* p) const { *p = v; }
    __device__ __forceinline__ double value() const { return v; }
};
struct AccF {
    float h, l;
    __device__ __forceinline__ static AccF zero() { return {0.0f, 0.0f}; }
    __device__ __forceinline__ static AccF load(const double* p) {
        const float2 f = *reinterpret_cast<const float2*>(p);
        return {f.x, f.y};
    }
    __device__ __forceinline__ static AccF load_cg(const double* p) {
        const float2 f = __ldcg(reinterpret_cast<const float2*>(p));
        return {f.x, f.y};
    }
    __device__ __forceinline__ void add(const AccF& b) {
        const float s = h + b.h, bv = s - h;
        float e = (h - (s - bv)) + (b.h - bv);
        e += l + b.l;
        h = s + e;
        l = e - (h - s);
    }
    __device__ __forceinline__ AccF shfl(int o) const {
        return {__shfl_xor_sync(0xffffffffu, h, o), __shfl_xor_sync(0xffffffffu, l, o)};
    }
    __device__ __forceinline__ void store(double* p) const { *reinterpret_cast<float2*>(p) = make_float2(h, l); }
    __device__ __forceinline__ double value() const { return (double)h + (double)l; }
};

// Warp sums of NPART_NR accumulators by recursive halving (as warp_store):
// on return lane 2k holds the warp total of value k in v[0].
template <typename A>
__device__ __forceinline__ A warp_halving(A (&v)[NPART_NR]) {
    const int lane = threadIdx.x & 31;
    A w[16];
#pragma unroll
    for (int k = 0; k < 16; k++) w[k] = k < NPART_NR ? v[k] : A::zero();
#pragma unroll
    for (int st = 0; st < 4; st++) {
        const int h = 8 >> st, o = 16 >> st;
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < h; j++) {
            const A send = up ? w[j] : w[j + h];
            A keep = up ? w[j + h] : w[j];
            keep.add(send.shfl(o));
            w[j] = keep;
        }
    }
    w[0].add(w[0].shfl(1));
    return w[0];
}

template <typename A>
__device__ __forceinline__ void macro_body_t(const MacroArgs& a, int bid) {
    Macro* m = a.macro;
    __shared__ A red[NPART_NR][8];
    __shared__ bool last;
    const int nb = a.nblk;
    const int per = (a.nrows + nb - 1) / nb;
    const int r0 = bid * per, r1 = min(a.nrows, r0 + per);
    A v[NPART_NR];
#pragma unroll
    for (int q = 0; q < NPART_NR; q++) v[q] = A::zero();
    for (int r = r0 + (int)threadIdx.x; r < r1; r += blockDim.x)
#pragma unroll
        for (int q = 0; q < NPART_NR; q++) v[q].add(A::load(a.part + (size_t)r * NPART_NR + q));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    {
        const A x = warp_halving<A>(v);
        if (!(lane & 1) && (lane >> 1) < NPART_NR) red[lane >> 1][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < NPART_NR) {
        A s = A::zero();
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s.add(red[threadIdx.x][w]);
        s.store(a.part2 + (size_t)bid * NPART_NR + threadIdx.x);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(a.ticket, 1u) == (unsigned)nb - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    // last block: one block row per thread, then the same fixed-order
    // warp/block tree as above, then the macro update
    __shared__ double tot[NPART_NR];
#pragma unroll
    for (int q = 0; q < NPART_NR; q++)
        v[q] = (int)threadIdx.x < nb ? A::load_cg(a.part2 + (size_t)threadIdx.x * NPART_NR + q) : A::zero();
    {
        const A x = warp_halving<A>(v);
        if (!(lane & 1) && (lane >> 1) < NPART_NR) red[lane >> 1][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < NPART_NR) {
        A t = A::zero();
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t.add(red[threadIdx.x][w]);
        tot[threadIdx.x] = t.value();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *a.ticket = 0;
        macro_update(a.cfg, m, tot);
    }
}

__device__ __forceinline__ void macro_body(const MacroArgs& a, int bid) {
    if (a.f32rows) macro_body_t<AccF>(a, bid);
    else macro_body_t<AccD>(a, bid);
}

__global__ void __launch_bounds__(256) k_macro(const __grid_constant__ MacroArgs a) {
    if (a.macro->done) return;
    macro_body(a, blockIdx.x);
}

__global__ void __launch_bounds__(256) kb_macro(const MacroArgs* __restrict__ tab, const int2* __restrict__ map) {
    const int2 m = map[blockIdx.x];
    const MacroArgs& a = tab[m.x];
    if (a.macro->done) return;
    macro_body(a, m.y);
}

// Increment head, first step: reset the macro state from the controls the
// host wrote into macro->ctl (one thread per RVE).
__device__ __forceinline__ void macro_begin(Macro* m) {
    const IncrCtl& c = m->ctl;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            m->dE[i][j] = 0.0;
            m->dE_acum[i][j] = 0.0;
        }
    for (int q = 0; q < 9; q++) {
        m->dE9[q] = 0.0;
        m->dE9_acc[q] = 0.0;
    }
    m->err_e = c.err0;
    m->err_s = c.err0;
    m->iter = 0;
    m->done = 0;
    m->converged = 0;
    m->status = 0;
    m->nr_iters = 0;
    m->tpass_drx = c.drx;
    m->e_vm = c.e_vm;
}

__global__ void k_macro_begin(Macro* m, int gate) {
    if (threadIdx.x == 0 && gate_open(m, gate)) macro_begin(m);
}

__global__ void kb_macro_begin(Macro* const* __restrict__ ms, int n, int gate) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && gate_open(ms[i], gate)) macro_begin(ms[i]);
}

__global__ void k_phase(Macro* m, int from, int to) {
    if (threadIdx.x == 0 && m->ctl.phase == from) m->ctl.phase = to;
}

// ------------------------------------------------------ increment head


// update_schmid (kinematics.c:430-463) and the rho-dependent products of the
// flow rule that stay fixed during an increment (constitutive.c:559-633).
// GND densities of voxel v: g1 = rho_g1 (screw), g2 = rho_g2 (edge type I),
// zero past n_sys; rho_g3 stays zero to first order.
__device__ __forceinline__ void load_gnd(const double* __restrict__ rho_g, int N, int v, int nsys,
                                         double g1[NS], double g2[NS]) {
#pragma unroll
    for (int j = 0; j < NS; j++) {
        g1[j] = (j < nsys) ? rho_g[(size_t)j * N + v] : 0.0;
        g2[j] = (j < nsys) ? rho_g[(size_t)(NS + j) * N + v] : 0.0;
    }
}

// rho_P and rho_F of system i with the projected GND densities
// (constitutive.c:558-577): sum_j Chi (Chi_1) times rho_s + |rho_g1 sin (cos)
// theta_g1| + |rho_g2 sin (cos) theta_g2|.
__device__ __forceinline__ void forest_parallel_gnd(const PhaseK<double>& P, const double* __restrict__ gp,
                                                    int i, const double rs[NS], const double g1[NS],
                                                    const double g2[NS], double& rP, double& rf) {
    rP = 0.0;
    rf = 0.0;
#pragma unroll
    for (int j = 0; j < NS; j++) {
        const int ij = i * NS + j;
        const double tf = rs[j] + fabs(g1[j] * gp[GP_COS1 + ij]) + fabs(g2[j] * gp[GP_COS2 + ij]);
        const double tp = rs[j] + fabs(g1[j] * gp[GP_SIN1 + ij]) + fabs(g2[j] * gp[GP_SIN2 + ij]);
        rP += P.chi[i][j] * tp;
        rf += P.chi1[i][j] * tf;
    }
}

// update_schmid and the flow-rule constants of one voxel (constitutive.c:
// 585-692 prefixes), in arithmetic type R: FP64, or FP32 for the FP32-bulk
// form, whose FP64 copies are then its FP32 values widened.
template <typename R>
__device__ __forceinline__ void begin_rates(const BeginArgs& a, int v, int ph, const PhaseK<R>& P) {
    const int N = a.g.N;
    const R drx = (R)a.macro->ctl.drx;
    R Rm[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) Rm[i][j] = (R)a.tranmat[(size_t)(3 * i + j) * N + v];
    for (int s = 0; s < P.n_sys; s++) {
        // R sym(n (x) b) R^T = sym(Rn (x) Rb): the rotated Schmid tensor from the
        // rotated slip normal and direction (kinematics.c:430-463 rotates the
        // tensor of Schm_xt, which is sym(n (x) b), init.c:205-212)
        R bs[3], ns[3], w[3][3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            bs[i] = Rm[i][0] * P.bb[s][0] + Rm[i][1] * P.bb[s][1] + Rm[i][2] * P.bb[s][2];
            ns[i] = Rm[i][0] * P.bn[s][0] + Rm[i][1] * P.bn[s][1] + Rm[i][2] * P.bn[s][2];
        }
#pragma unroll
        for (int i = 0; i < 3; i++) w[i][i] = ns[i] * bs[i];
        w[1][2] = w[2][1] = (R)0.5 * (ns[1] * bs[2] + ns[2] * bs[1]);
        w[0][2] = w[2][0] = (R)0.5 * (ns[0] * bs[2] + ns[2] * bs[0]);
        w[0][1] = w[1][0] = (R)0.5 * (ns[0] * bs[1] + ns[1] * bs[0]);
        R o6[6];
        sym_to_b6<R>(w, o6);
#pragma unroll
        for (int q = 0; q < 5; q++) {
            a.schm64[(size_t)(s * 5 + q) * N + v] = (double)o6[q];
            if (a.schm32) a.schm32[(size_t)(s * 5 + q) * N + v] = (float)o6[q];
        }
    }
    R rs[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) rs[i] = (i < P.n_sys) ? (R)a.rho_s[(size_t)i * N + v] : (R)0;
    // GND densities enter the FP64 form of the constants only (an FP32-bulk
    // context with GND computes them in FP64)
    double g1[NS], g2[NS];
    const double* gp = a.rho_g ? a.gproj + (size_t)(ph - 1) * GP_STRIDE : nullptr;
    if constexpr (sizeof(R) == 8)
        if (gp) load_gnd(a.rho_g, N, v, P.n_sys, g1, g2);
    for (int i = 0; i < P.n_sys; i++) {
        R rP = (R)0, rf = (R)0;
        bool done = false;
        if constexpr (sizeof(R) == 8)
            if (gp) {
                forest_parallel_gnd(P, gp, i, rs, g1, g2, rP, rf);
                done = true;
            }
        if (!done) {
#pragma unroll
            for (int j = 0; j < NS; j++) {
                rP += P.chi[i][j] * rs[j];
                rf += P.chi1[i][j] * rs[j];
            }
        }
        const R rm_stale = (R)a.rho_m[(size_t)i * N + v];
        const R rm = P.k_rhom[i] * sqrt(rP * rf);
        const R tp = P.k_tpass[i] * sqrt(fabs(rP + rm)) + drx;
        const R tps = P.k_tpass[i] * sqrt(fabs(rP + rm_stale)) + drx;
        const R itc = (R)1 / (P.tau0 + P.k_tcut[i] * sqrt(rf));
        const R go = P.k_gamo[i] * rm / sqrt(rf);
        const R f4[4] = {tp, itc, go, tps};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            a.fc64[(size_t)(12 * q + i) * N + v] = (double)f4[q];
            if (a.fc32) a.fc32[(size_t)(12 * q + i) * N + v] = (float)f4[q];
        }
        // the voxel's NR constant record of this system, both 16-byte halves
        // together (a whole 32-byte sector): the Schmid vector stored above by
        // this thread, passing stress, 1/(tau0 + tau_cut), gamma0_dot
        if (a.nrc32) {
            const float* sc = a.schm32 + (size_t)(i * 5) * N + v;
            *reinterpret_cast<float4*>(a.nrc32 + nrc_index(v, i, 0)) = make_float4(sc[0], sc[N], sc[2 * (size_t)N], sc[3 * (size_t)N]);
            *reinterpret_cast<float4*>(a.nrc32 + nrc_index(v, i, 1)) =
                make_float4(sc[4 * (size_t)N], (float)f4[0], (float)f4[1], (float)f4[2]);
        }
    }
}

// R: arithmetic type of the Schmid vectors and flow constants (float in the
// FP32-bulk form without GND, else double); one kernel per type keeps the
// FP32 kernel's registers its own.
template <typename R>
__device__ __forceinline__ void begin_body(const BeginArgs& a, int bid) {
    const int v = bid * 128 + threadIdx.x;
    const int N = a.g.N;
    if (v >= N) return;
    const IncrCtl& ctl = a.macro->ctl;
    const int creep = ctl.creep;
#pragma unroll
    for (int c = 0; c < 9; c++) {
        const double d = a.dg64[(size_t)c * N + v];
        a.dg_old[(size_t)c * N + v] = d;
        a.dg64[(size_t)c * N + v] = creep ? ctl.dgavg9[c] : d + ctl.udot9[c];
    }
    const int ph = a.phase[v];
    const PhaseK<double>& P = a.mat.ph[ph - 1];
    // the deferred antisymmetric spectrum starts the increment at zero
    if (a.acc)
        for (int i = v; i < a.acc_floats; i += N) a.acc[i] = 0.0f;
    if (a.b6_32) {
#pragma unroll
        for (int c = 0; c < 6; c++) {
            a.b6_32[(size_t)c * N + v] = (float)(a.epsp[(size_t)c * N + v] - a.dg64[(size_t)c * N + v]);
            a.ddg32[(size_t)c * N + v] = 0.0f;
        }
#pragma unroll
        for (int c = 6; c < 9; c++) a.ddg32[(size_t)c * N + v] = 0.0f;
    }
    if (!a.mat.ph[ph - 1].crystal) return;
    if constexpr (sizeof(R) == 4) begin_rates<float>(a, v, ph, a.ph32[ph - 1]);
    else begin_rates<double>(a, v, ph, P);
}

// Register budget of the FP32 head: twelve blocks per SM (40 registers, 16
// bytes spilled, 48 warps per SM instead of 32); the FP64 head keeps its own.
template <typename R> struct BeginMinBlocks { static constexpr int v = 1; };
template <> struct BeginMinBlocks<float> { static constexpr int v = 12; };

template <typename R>
__global__ void __launch_bounds__(128, BeginMinBlocks<R>::v) k_begin(const __grid_constant__ BeginArgs a) {
    if (!gate_open(a.macro, a.gate)) return;
    begin_body<R>(a, blockIdx.x);
}

template <typename R>
__global__ void __launch_bounds__(128, BeginMinBlocks<R>::v) kb_begin(const BeginArgs* __restrict__ tab, const int2* __restrict__ map) {
    const int2 m = map[blockIdx.x];
    const BeginArgs& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    begin_body<R>(a, m.y);
}

// FP32 bulk: fold the FP32 displacement-gradient increment into the FP64
// field and seed the FP64 refinement with the FP32 stress.

__device__ __forceinline__ void fold_body(const FoldArgs& a, int bid) {
    const int v = bid * 256 + threadIdx.x;
    const int N = a.g.N;
    if (v >= N) return;
#pragma unroll
    for (int c = 0; c < 9; c++) a.dg64[(size_t)c * N + v] += (double)a.ddg32[(size_t)c * N + v];
#pragma unroll
    for (int c = 0; c < 6; c++) a.sig64[(size_t)c * N + v] = (double)a.sig32[(size_t)c * N + v];
}

__global__ void __launch_bounds__(256) k_fold(const __grid_constant__ FoldArgs a) {
    if (!gate_open(a.macro, a.gate)) return;
    fold_body(a, blockIdx.x);
}

__global__ void __launch_bounds__(256) kb_fold(const FoldArgs* __restrict__ tab, const int2* __restrict__ map) {
    const int2 m = map[blockIdx.x];
    const FoldArgs& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    fold_body(a, m.y);
}

// ------------------------------------------------------ increment tail


// Orientation (constitutive.c:142-194): Rodrigues-type update of R by the
// rotation increment rot (the reference drops rotations below 1e-6 by
// rescaling with tan(|w|/2) before resetting |w| to 1).
__device__ void reorient(double tran[3][3], const double rot[3][3]) {
    double w[3] = {rot[2][1], rot[0][2], rot[1][0]};
    double wn = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    double wt = tan(wn / 2.0);
    if (fabs(wn) < 1E-6) wn = 1.0;
    for (int i = 0; i < 3; i++) w[i] *= wt / wn;
    const double om[3][3] = {{0., -w[2], w[1]}, {w[2], 0., -w[0]}, {-w[1], w[0], 0.}};
    double om2[3][3], r[3][3], tn[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) om2[i][j] = om[i][0] * om[0][j] + om[i][1] * om[1][j] + om[i][2] * om[2][j];
    wt = wt * wt;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r[i][j] = (double)(i == j) + 2. * (om[i][j] + om2[i][j]) / (1. + wt);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) tn[i][j] = r[i][0] * tran[0][j] + r[i][1] * tran[1][j] + r[i][2] * tran[2][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) tran[i][j] = tn[i][j];
}

// The same update from an FP32 rotation increment: the small part
// D = 2 (om + om^2) / (1 + wt^2) of r = I + D in FP32, tran += D tran with the
// sum in FP64 (D is of the order of the rotation, so its FP32 rounding is far
// below the FP64 resolution of tran's entries).
__device__ void reorient(double tran[3][3], const float rot[3][3]) {
    float w[3] = {rot[2][1], rot[0][2], rot[1][0]};
    float wn = sqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    float wt = tanf(wn / 2.0f);
    if (fabsf(wn) < 1E-6f) wn = 1.0f;
    for (int i = 0; i < 3; i++) w[i] *= wt / wn;
    const float om[3][3] = {{0.f, -w[2], w[1]}, {w[2], 0.f, -w[0]}, {-w[1], w[0], 0.f}};
    float d[3][3];
    const float sc = 2.f / (1.f + wt * wt);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            d[i][j] = sc * (om[i][j] + om[i][0] * om[0][j] + om[i][1] * om[1][j] + om[i][2] * om[2][j]);
    double tn[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            tn[i][j] = tran[i][j] + (double)(d[i][0] * (float)tran[0][j] + d[i][1] * (float)tran[1][j] +
                                             d[i][2] * (float)tran[2][j]);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) tran[i][j] = tn[i][j];
}

// One directional derivative of Gradient_ShearRate (constitutive.c:881-1112)
// from the same-grain bits of the plus and minus neighbours: backward,
// forward or central difference, zero with no neighbour in the grain.
__device__ __forceinline__ double gb_diff(double c, double vp, double vm, unsigned same_p, unsigned same_m) {
    if (!same_p && same_m) return c - vm;
    if (same_p && !same_m) return vp - c;
    if (same_p && same_m) return (vp - vm) / 2.0;
    return 0.0;
}

// gadot_grad of system i at voxel v (one rank: periodic neighbours).
__device__ __forceinline__ void slip_rate_gradient(const EndArgs& a, int v, int i, double gr[3]) {
    const int n0 = a.g.n0, n1 = a.g.n1, n2 = a.g.n2;
    const int x = v / (n1 * n2), y = (v / n2) % n1, z = v % n2;
    const int xp = x + 1 == n0 ? 0 : x + 1, xm = x == 0 ? n0 - 1 : x - 1;
    const int yp = y + 1 == n1 ? 0 : y + 1, ym = y == 0 ? n1 - 1 : y - 1;
    const int zp = z + 1 == n2 ? 0 : z + 1, zm = z == 0 ? n2 - 1 : z - 1;
    const double* gd = a.gamdot + (size_t)i * a.g.N;
    const unsigned m = a.gbm[v];
    gr[0] = gb_diff(gd[v], gd[(xp * n1 + y) * n2 + z], gd[(xm * n1 + y) * n2 + z], m & 1u, m & 2u);
    gr[1] = gb_diff(gd[v], gd[(x * n1 + yp) * n2 + z], gd[(x * n1 + ym) * n2 + z], m & 4u, m & 8u);
    gr[2] = gb_diff(gd[v], gd[(x * n1 + y) * n2 + zp], gd[(x * n1 + y) * n2 + zm], m & 16u, m & 32u);
}

// update_orient and DislocationEvolution of one crystal voxel in arithmetic
// type R (FP64, or FP32 for the FP32-bulk form without GND: the rates in
// FP32, the state updates -- rho_s, gam_acum, the orientation -- added in
// FP64). q: the block's partial sums.
template <typename R>
__device__ __forceinline__ void end_crystal(const EndArgs& a, int v, int ph, const PhaseK<R>& P, const double (&vg)[9],
                                            double (&q)[NPART_END]) {
    const int N = a.g.N;
    const double dt = a.mat.dt;
    const int reorient_on = a.macro->ctl.tail & 1;
    const int grad_on = a.macro->ctl.tail & 2;
    R gd[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) gd[i] = (i < P.n_sys) ? (R)a.gamdot[(size_t)i * N + v] : (R)0;
    if (reorient_on) {
        // update_orient (constitutive.c:196-273)
        double tr[3][3];
        R trr[3][3], Lp[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, rot[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                tr[i][j] = a.tranmat[(size_t)(3 * i + j) * N + v];
                trr[i][j] = (R)tr[i][j];
            }
        for (int s = 0; s < P.n_sys; s++) {
            R bs[3], ns[3];
            for (int i = 0; i < 3; i++) {
                bs[i] = trr[i][0] * P.bb[s][0] + trr[i][1] * P.bb[s][1] + trr[i][2] * P.bb[s][2];
                ns[i] = trr[i][0] * P.bn[s][0] + trr[i][1] * P.bn[s][1] + trr[i][2] * P.bn[s][2];
            }
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) Lp[i][j] += bs[i] * ns[j] * gd[s];
        }
        // antisymmetric VelGrad: A12 = vg[6], A13 = vg[7], A23 = vg[8]
        const R rl[3][3] = {{(R)0, (R)vg[6], (R)vg[7]}, {-(R)vg[6], (R)0, (R)vg[8]}, {-(R)vg[7], -(R)vg[8], (R)0}};
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                rot[i][j] = ((R)a.udot_a[i][j] + rl[i][j] - (Lp[i][j] - Lp[j][i]) / (R)2) * (R)dt;
        reorient(tr, rot);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) a.tranmat[(size_t)(3 * i + j) * N + v] = tr[i][j];
    }
    // DislocationEvolution (constitutive.c:1373-1426), with rho_F and
    // rho_m of the increment's flow-rule calls and the stored rho_m
    // (the value before this increment) in rho_tot.
    double rs64[NS];
    R rs[NS], rf[NS], rP[NS], rm[NS], rtot = (R)0;
#pragma unroll
    for (int i = 0; i < NS; i++) {
        rs64[i] = (i < P.n_sys) ? a.rho_s[(size_t)i * N + v] : 0.0;
        rs[i] = (R)rs64[i];
    }
    // GND densities before this increment's update (the flow rule's
    // trial values and rho_tot, evolution.c:1041-1045); FP64 form only
    double g1[NS], g2[NS];
    const double* gp = a.rho_g ? a.gproj + (size_t)(ph - 1) * GP_STRIDE : nullptr;
    if constexpr (sizeof(R) == 8)
        if (gp) load_gnd(a.rho_g, N, v, P.n_sys, g1, g2);
    for (int i = 0; i < P.n_sys; i++) {
        R x = (R)0, y = (R)0;
        bool done = false;
        if constexpr (sizeof(R) == 8)
            if (gp) {
                forest_parallel_gnd(P, gp, i, rs, g1, g2, x, y);
                done = true;
            }
        if (!done) {
#pragma unroll
            for (int j = 0; j < NS; j++) {
                x += P.chi[i][j] * rs[j];
                y += P.chi1[i][j] * rs[j];
            }
        }
        rP[i] = x;
        rf[i] = y;
        rm[i] = P.k_rhom[i] * sqrt(x * y);
        const R rmo = (R)a.rho_m[(size_t)i * N + v];
        if constexpr (sizeof(R) == 8)
            rtot += gp ? rs[i] + rmo + sqrt(g1[i] * g1[i] + g2[i] * g2[i]) : rs[i] + rmo;
        else
            rtot += rs[i] + rmo;
    }
    R s6[6];
#pragma unroll
    for (int c = 0; c < 6; c++) s6[c] = (R)a.sig64[(size_t)c * N + v];
    const R eqb = exp(-(R)1 * P.q_bulk);
    const R dtr = (R)dt;
    // the voxel's sums of q[0, 1, 3..6] in type R (q[2] takes the FP64 rho_s)
    R qa[7] = {(R)0, (R)0, (R)0, (R)0, (R)0, (R)0, (R)0};
    for (int i = 0; i < P.n_sys; i++) {
        // Schmid vectors: the FP32 copy in the FP32 form (its FP64 copy is the
        // same values widened)
        R sc[5];
#pragma unroll
        for (int k = 0; k < 5; k++) {
            if constexpr (sizeof(R) == 4) sc[k] = a.schm32[(size_t)(i * 5 + k) * N + v];
            else sc[k] = a.schm64[(size_t)(i * 5 + k) * N + v];
        }
        const R rss = sc[0] * s6[0] + sc[1] * s6[1] + sc[2] * s6[2] + sc[3] * s6[3] + sc[4] * s6[4];
        const R b = P.burgers[i];
        const R den = fabs(rss) + (R)1.0E-4;
        const R ddip = P.k_ddip[i] / den;
        const R hyd = P.k_hydr[i] * den;  // k_hyd / ddip
        const R clim = (R)1E-17 * rtot * (R)0.5 * (R)1E24 * ddip * P.k_d0b[i] * (rs[i] * rs[i]) *
                       (exp(fabs(hyd) * P.k_hexp[i]) - (R)1) * eqb;
        const R ag = fabs(gd[i]);
        const R sq = sqrt(rf[i]);
        qa[4] += clim * dtr;
        qa[5] += ag * (P.c4 * sq) * dtr;
        qa[6] += ag * (P.c5 * rs[i]) * dtr;
        const R dot = ag * (P.c4 * sq + P.c6 * ddip * rm[i] - P.c5 * rs[i]) - clim;
        // the state update in FP64 (the same expression in the FP64 form)
        const double rn = rs64[i] + (double)dot * dt;
        a.rho_s[(size_t)i * N + v] = rn;
        a.rho_m[(size_t)i * N + v] = (double)rm[i];
        a.gam_acum[(size_t)i * N + v] += (double)gd[i] * dt;
        if constexpr (sizeof(R) == 8)
            if (gp) {
                // first-order GND rates (constitutive.c:1428-1522): screw
                // grad(gamdot).p / b / L0, edge type I -grad(gamdot).b / b / L0
                double gr[3] = {0.0, 0.0, 0.0};
                if (grad_on) slip_rate_gradient(a, v, i, gr);
                const double* bp = gp + GP_BP + 3 * i;
                const double d1 = (gr[0] * bp[0] + gr[1] * bp[1] + gr[2] * bp[2]) / b / a.l0;
                const double d2 =
                    -1.0 * (gr[0] * P.bb[i][0] + gr[1] * P.bb[i][1] + gr[2] * P.bb[i][2]) / b / a.l0;
                const double n1 = g1[i] + d1 * dt, n2 = g2[i] + d2 * dt;
                a.rho_g[(size_t)i * N + v] = n1;
                a.rho_g[(size_t)(NS + i) * N + v] = n2;
                q[18] += sqrt(n1 * n1 + n2 * n2);
            }
        qa[0] += rf[i];
        qa[1] += rP[i];
        q[2] += rn;
        qa[3] += rm[i];
    }
    q[0] += (double)qa[0];
    q[1] += (double)qa[1];
#pragma unroll
    for (int k = 3; k < 7; k++) q[k] += (double)qa[k];
}

// R as in the head: float in the FP32-bulk form without GND, else double.
template <typename R>
__device__ __forceinline__ void end_body(const EndArgs& a, int bid) {
    const int v = bid * END_BLOCK + threadIdx.x;
    const int N = a.g.N;
    const double dt = a.mat.dt;
    constexpr bool r32 = sizeof(R) == 4;
    double q[NPART_END];
#pragma unroll
    for (int i = 0; i < NPART_END; i++) q[i] = 0.0;
    if (v < N) {
        // VelGrad = (DisGrad - DisGrad_old)/dt (evolution.c:1268-1272); the
        // FP32-bulk form multiplies by 1/dt
        double vg[9];
        const double idt = 1.0 / dt;
#pragma unroll
        for (int c = 0; c < 9; c++) {
            const double d = a.dg64[(size_t)c * N + v] - a.dg_old[(size_t)c * N + v];
            vg[c] = r32 ? d * idt : d / dt;
            a.dg_old[(size_t)c * N + v] = vg[c];
        }
        // Eps += Edot dt (evolution.c:1297-1301)
        double ep[6], ed[5];
#pragma unroll
        for (int c = 0; c < 5; c++) ed[c] = a.edot[(size_t)c * N + v];
#pragma unroll
        for (int c = 0; c < 6; c++) {
            ep[c] = a.epsp[(size_t)c * N + v] + (c < 5 ? ed[c] * dt : 0.0);
            a.epsp[(size_t)c * N + v] = ep[c];
            q[7 + c] = ep[c];
        }
#pragma unroll
        for (int c = 0; c < 5; c++) q[13 + c] = ed[c];
        if (a.sig32)
#pragma unroll
            for (int c = 0; c < 6; c++) a.sig32[(size_t)c * N + v] = (float)a.sig64[(size_t)c * N + v];
        const int ph = a.phase[v];
        if (a.mat.ph[ph - 1].crystal) {
            if constexpr (r32) end_crystal<float>(a, v, ph, a.ph32[ph - 1], vg, q);
            else end_crystal<double>(a, v, ph, a.mat.ph[ph - 1], vg, q);
        }
    }
    block_reduce_store<NPART_END>(q, a.part + (size_t)bid * NPART_END);
}

template <typename R>
// Register budget of six blocks per SM: 80 registers (48 bytes spilled)
// instead of 96, 24 instead of 20 warps per SM; FP32-bulk tail 1.71 -> 1.52 ms
// at 128^3.
__global__ void __launch_bounds__(END_BLOCK, 6) k_end(const __grid_constant__ EndArgs a) {
    if (!gate_open(a.macro, a.gate)) return;
    end_body<R>(a, blockIdx.x);
}

template <typename R>
__global__ void __launch_bounds__(END_BLOCK, 6) kb_end(const EndArgs* __restrict__ tab, const int2* __restrict__ map) {
    const int2 m = map[blockIdx.x];
    const EndArgs& a = tab[m.x];
    if (!gate_open(a.macro, a.gate)) return;
    end_body<R>(a, m.y);
}


// AvgDislocation (constitutive.c:1681-1808) and <Eps>, <Edot>
// (evolution.c:1307-1323), in the B basis.
__device__ __forceinline__ void end_reduce_body(const EndReduceArgs& a) {
    double v[NPART_END];
#pragma unroll
    for (int q = 0; q < NPART_END; q++) v[q] = 0.0;
    for (int b = threadIdx.x; b < a.nblocks; b += blockDim.x)
#pragma unroll
        for (int q = 0; q < NPART_END; q++) v[q] += a.part[(size_t)b * NPART_END + q];
    __shared__ double tot[NPART_END];
    double o[NPART_END];
    block_reduce_store<NPART_END>(v, o);
    if (threadIdx.x < NPART_END) tot[threadIdx.x] = o[threadIdx.x];
    __syncthreads();
    if (threadIdx.x != 0) return;
    Macro* m = a.macro;
    m->rho_dip_acc += tot[4];
    m->rho_for_acc += tot[5];
    m->rho_inp_acc += tot[6];
    m->rho_avg[0] = tot[0] * a.wgt;
    m->rho_avg[1] = tot[1] * a.wgt;
    m->rho_avg[2] = tot[2] * a.wgt;
    m->rho_avg[3] = tot[3] * a.wgt;
    m->rho_avg[4] = tot[18] * a.wgt;
    m->rho_avg[5] = m->rho_dip_acc * a.wgt;
    m->rho_avg[6] = m->rho_for_acc * a.wgt;
    m->rho_avg[7] = m->rho_inp_acc * a.wgt;
    for (int c = 0; c < 6; c++) m->eps_avg6[c] = tot[7 + c] * a.wgt;
    for (int c = 0; c < 5; c++) m->edot_avg6[c] = tot[13 + c] * a.wgt;
    m->edot_avg6[5] = 0.0;
}

__global__ void __launch_bounds__(256) k_end_reduce(const __grid_constant__ EndReduceArgs a) {
    if (!gate_open(a.macro, a.gate)) return;
    end_reduce_body(a);
}

// one block per RVE
__global__ void __launch_bounds__(256) kb_end_reduce(const EndReduceArgs* __restrict__ tab) {
    const EndReduceArgs& a = tab[blockIdx.x];
    if (!gate_open(a.macro, a.gate)) return;
    end_reduce_body(a);
}

// ------------------------------------------------------------- launchers

template <typename T>
static void nr_set(Ctx& c, NrSet<T>& S, const Material<T>& mat, T* sig, const T* dg, const T* epsb,
                   const T* schm, const T* fc, const T* sgr, T* edot, T* gamdot, T tol, int stale_mode,
                   int gate) {
    NrArgs<T>& a = S.a;
    a.mat = mat;
    a.g = c.g;
    a.sig = sig; a.dg = dg; a.epsb = epsb; a.schm = schm; a.fc = fc;
    a.nrc = sizeof(T) == 4 ? c.nrc32 : nullptr;
    a.orient = c.orient; a.phase = c.phase; a.sgr = sgr; a.edot = edot; a.gamdot = gamdot;
    a.macro = c.macro; a.part = c.part_nr; a.tol = tol; a.itmax = c.nr_itmax;
    a.nr_mode = c.nr_mode; a.stale_mode = stale_mode; a.gate = gate;
    a.quick_accept = 0;
    a.mixed = 0;
    S.grid = c.nb_nr;
}

void build_solver_sets(Ctx& c) {
    KernelSets& k = *c.ks;
    if (c.precision == 0) {
        nr_set<double>(c, k.nr64, c.m64, c.sig64, c.dg64, c.epsp, c.schm64, c.fc64, c.sgr64, c.edot64,
                       c.gamdot64, (double)c.nr_tol64, 1, GATE_RUNNING);
    } else {
        // FP64 refinement at the end of the loop: no stale rho_m, runs once
        nr_set<double>(c, k.nr64, c.m64, c.sig64, c.dg64, c.epsp, c.schm64, c.fc64, c.sgr64, c.edot64,
                       c.gamdot64, (double)c.nr_tol64, 0, GATE_ENDING);
        nr_set<float>(c, k.nr32, c.m32, c.sig32, c.ddg32, c.b6_32, c.schm32, c.fc32, c.sgr32, nullptr,
                      nullptr, (float)c.nr_tol32, 1, GATE_RUNNING);
        k.nr32.a.quick_accept = 1;
        // the refinement starts from the converged FP32 stress: its last step
        // is below the tolerance, and the slip rates it keeps are those of the
        // evaluation before that step (a change below the NR tolerance)
        k.nr64.a.quick_accept = 1;
        // corrections with the FP32 Jacobian of the FP32 constant records
        k.nr64.a.mixed = 1;
        k.nr64.a.nrc = c.nrc32;
    }
    MacroArgs& m = k.mac;
    m.cfg = c.cfg; m.macro = c.macro; m.part = c.part_nr; m.nrows = c.nb_nr * (NR_BLOCK / 32);
    m.part2 = c.part_nr2; m.ticket = c.ticket; m.f32rows = c.precision != 0;
    // first-level blocks: ~32 warp rows each, at most MACRO_BLOCKS (a small RVE
    // does not pay for 64 blocks with a fence and a ticket each)
    m.nblk = m.nrows / 32 < 1 ? 1 : (m.nrows / 32 > MACRO_BLOCKS ? MACRO_BLOCKS : m.nrows / 32);
    BeginArgs& b = k.beg;
    b.mat = c.m64; b.g = c.g; b.macro = c.macro; b.gate = GATE_BEGIN;
    b.dg64 = c.dg64; b.dg_old = c.dg_old; b.tranmat = c.tranmat; b.rho_s = c.rho_s;
    b.rho_m = c.rho_m; b.phase = c.phase; b.schm64 = c.schm64; b.fc64 = c.fc64;
    b.schm32 = c.schm32; b.fc32 = c.fc32; b.b6_32 = c.b6_32; b.ddg32 = c.ddg32; b.epsp = c.epsp;
    b.nrc32 = c.nrc32;
    b.acc = c.precision != 0 && c.ks->s32.defer ? reinterpret_cast<float*>(c.spec) + 18 * (size_t)c.g.Nh : nullptr;
    b.acc_floats = (int)(6 * (size_t)c.g.Nh);
    b.rho_g = c.rho_g; b.gproj = c.gproj;
    for (int p = 0; p < 2; p++) b.ph32[p] = c.m32.ph[p];
    k.grid_begin = (c.g.N + 127) / 128;
    FoldArgs& f = k.fold;
    f.g = c.g; f.macro = c.macro; f.gate = GATE_ENDING; f.dg64 = c.dg64; f.ddg32 = c.ddg32;
    f.sig64 = c.sig64; f.sig32 = c.sig32;
    k.grid_fold = (c.g.N + 255) / 256;
    EndArgs& e = k.end;
    e.mat = c.m64; e.g = c.g; e.macro = c.macro; e.gate = GATE_ENDING;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) e.udot_a[i][j] = c.udot_a[i][j];
    e.dg_old = c.dg_old; e.dg64 = c.dg64; e.epsp = c.epsp; e.edot = c.edot64;
    e.tranmat = c.tranmat; e.rho_s = c.rho_s; e.rho_m = c.rho_m; e.gamdot = c.gamdot64;
    e.gam_acum = c.gam_acum; e.sig64 = c.sig64; e.schm64 = c.schm64; e.phase = c.phase;
    e.sig32 = c.sig32; e.part = c.part_end;
    e.rho_g = c.rho_g; e.gproj = c.gproj; e.gbm = c.gbm; e.l0 = c.l0;
    e.schm32 = c.schm32;
    for (int p = 0; p < 2; p++) e.ph32[p] = c.m32.ph[p];
    k.grid_end = c.nb_end;
    EndReduceArgs& r = k.endr;
    r.macro = c.macro; r.gate = GATE_ENDING; r.part = c.part_end; r.nblocks = c.nb_end; r.wgt = c.cfg.wgt;
}

// FP32 sweeps: the block's constant records and the copy barrier; FP64
// sweeps: the per-element staging columns and the slip-rate columns
template <typename T> static constexpr size_t nr_smem() {
    return sizeof(T) == 4 ? (size_t)NRC_BLOCK_FLOATS * sizeof(float) + 16
                          : (size_t)(NSTAGE + NS) * NR_BLOCK * sizeof(T);
}
template <typename T> static constexpr size_t nrb_smem() { return nr_smem<T>() + 72 * sizeof(T); }

template <typename T> static void nr_attributes() {
    cudaFuncSetAttribute(k_nr<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nr_smem<T>());
    cudaFuncSetAttribute(k_nr<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nr_smem<T>());
    cudaFuncSetAttribute(kb_nr<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nrb_smem<T>());
    cudaFuncSetAttribute(kb_nr<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nrb_smem<T>());
}

void solver_attributes() {
    nr_attributes<double>();
    nr_attributes<float>();
}

template <typename T>
static cudaError_t nr_launch(Ctx& c, const NrSet<T>& S, int gate, int grp) {
    NrArgs<T> a = S.a;
    a.gate = gate;
    prof_mark(c, grp, true);
    if (c.nr_mode) k_nr<T, 1><<<S.grid, NR_BLOCK, nr_smem<T>(), c.stream>>>(a);
    else k_nr<T, 0><<<S.grid, NR_BLOCK, nr_smem<T>(), c.stream>>>(a);
    prof_mark(c, grp, false);
    return cudaGetLastError();
}

cudaError_t launch_nr(Ctx& c, int refine, int gate) {
    const KernelSets& k = *c.ks;
    if (c.precision == 0) return nr_launch<double>(c, k.nr64, gate, PG_NR);
    if (refine) return nr_launch<double>(c, k.nr64, gate, PG_REFINE);
    return nr_launch<float>(c, k.nr32, gate, PG_NR);
}

cudaError_t launch_macro(Ctx& c) {
    prof_mark(c, PG_MACRO, true);
    k_macro<<<c.ks->mac.nblk, 256, 0, c.stream>>>(c.ks->mac);
    prof_mark(c, PG_MACRO, false);
    return cudaGetLastError();
}

cudaError_t launch_macro_begin(Ctx& c, int gate) {
    c.launches++;
    k_macro_begin<<<1, 32, 0, c.stream>>>(c.macro, gate);
    return cudaGetLastError();
}

cudaError_t launch_phase(Ctx& c, int from, int to) {
    c.launches++;
    k_phase<<<1, 32, 0, c.stream>>>(c.macro, from, to);
    return cudaGetLastError();
}

bool head_tail_fp32(const Ctx& c) { return c.precision != 0 && !c.rho_g; }

cudaError_t launch_begin(Ctx& c, int gate) {
    BeginArgs a = c.ks->beg;
    a.gate = gate;
    prof_mark(c, PG_BEGIN, true);
    if (head_tail_fp32(c)) k_begin<float><<<c.ks->grid_begin, 128, 0, c.stream>>>(a);
    else k_begin<double><<<c.ks->grid_begin, 128, 0, c.stream>>>(a);
    prof_mark(c, PG_BEGIN, false);
    return cudaGetLastError();
}

cudaError_t launch_fold(Ctx& c, int gate) {
    const cudaError_t e = launch_spectral_flush(c, gate);
    if (e != cudaSuccess) return e;
    FoldArgs a = c.ks->fold;
    a.gate = gate;
    c.launches++;
    k_fold<<<c.ks->grid_fold, 256, 0, c.stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_end(Ctx& c, int gate) {
    EndArgs a = c.ks->end;
    a.gate = gate;
    prof_mark(c, PG_END, true);
    if (head_tail_fp32(c)) k_end<float><<<c.ks->grid_end, END_BLOCK, 0, c.stream>>>(a);
    else k_end<double><<<c.ks->grid_end, END_BLOCK, 0, c.stream>>>(a);
    prof_mark(c, PG_END, false);
    EndReduceArgs r = c.ks->endr;
    r.gate = gate;
    c.launches++;
    k_end_reduce<<<1, 256, 0, c.stream>>>(r);
    return cudaGetLastError();
}

// ---- batched launchers (tables built by the batch; gates inside the tables)

cudaError_t launch_nr_batch(int precision, int nr_mode, const BatchLaunch& L, cudaStream_t st) {
    if (precision == 0) {
        if (nr_mode) kb_nr<double, 1><<<L.nblk, NR_BLOCK, nrb_smem<double>(), st>>>((const NrArgs<double>*)L.tab, L.map);
        else kb_nr<double, 0><<<L.nblk, NR_BLOCK, nrb_smem<double>(), st>>>((const NrArgs<double>*)L.tab, L.map);
    } else {
        if (nr_mode) kb_nr<float, 1><<<L.nblk, NR_BLOCK, nrb_smem<float>(), st>>>((const NrArgs<float>*)L.tab, L.map);
        else kb_nr<float, 0><<<L.nblk, NR_BLOCK, nrb_smem<float>(), st>>>((const NrArgs<float>*)L.tab, L.map);
    }
    return cudaGetLastError();
}

cudaError_t launch_macro_batch(const BatchLaunch& L, cudaStream_t st) {
    kb_macro<<<L.nblk, 256, 0, st>>>((const MacroArgs*)L.tab, L.map);
    return cudaGetLastError();
}

int launch_begin_batch(const BatchLaunch* L, cudaStream_t st) {
    const BatchLaunch& mb = L[BL_MBEGIN];
    kb_macro_begin<<<(mb.nblk + 127) / 128, 128, 0, st>>>((Macro* const*)mb.tab, mb.nblk, GATE_BEGIN);
    int n = 1;
    const BatchLaunch &b = L[BL_BEGIN], &b32 = L[BL_BEGIN32];
    if (b.nblk) {
        kb_begin<double><<<b.nblk, 128, 0, st>>>((const BeginArgs*)b.tab, b.map);
        n++;
    }
    if (b32.nblk) {
        kb_begin<float><<<b32.nblk, 128, 0, st>>>((const BeginArgs*)b32.tab, b32.map);
        n++;
    }
    return n;
}

int launch_end_batch(int precision, int nr_mode, const BatchLaunch* L, cudaStream_t st) {
    int n = 1;
    if (precision != 0) {
        n += launch_flush_batch(L, st);
        const BatchLaunch& f = L[BL_FOLD];
        kb_fold<<<f.nblk, 256, 0, st>>>((const FoldArgs*)f.tab, f.map);
        const BatchLaunch& r = L[BL_REFINE];
        if (nr_mode) kb_nr<double, 1><<<r.nblk, NR_BLOCK, nrb_smem<double>(), st>>>((const NrArgs<double>*)r.tab, r.map);
        else kb_nr<double, 0><<<r.nblk, NR_BLOCK, nrb_smem<double>(), st>>>((const NrArgs<double>*)r.tab, r.map);
        n += 2;
    }
    const BatchLaunch &e = L[BL_END], &e32 = L[BL_END32];
    if (e.nblk) {
        kb_end<double><<<e.nblk, END_BLOCK, 0, st>>>((const EndArgs*)e.tab, e.map);
        n++;
    }
    if (e32.nblk) {
        kb_end<float><<<e32.nblk, END_BLOCK, 0, st>>>((const EndArgs*)e32.tab, e32.map);
        n++;
    }
    const BatchLaunch& er = L[BL_ENDR];
    kb_end_reduce<<<er.nblk, 256, 0, st>>>((const EndReduceArgs*)er.tab);
    return n;
}

}  // namespace evpg
