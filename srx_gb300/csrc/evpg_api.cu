// C ABI of include/evpg.h: context set-up, state transfer and the
// equilibrium-loop orchestration on the context's stream.
#include "evpg.h"
#include "evpg_ctx.h"
#include "evpg_plan.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <vector>

namespace evpg {

static thread_local char g_err[512] = "";

static int fail(int st, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return st;
}

int record_error(int st, const char* msg) {
    snprintf(g_err, sizeof g_err, "%s", msg);
    return st;
}

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return fail(EVPG_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                            \
    } while (0)

// ------------------------------------------------------------- materials

template <typename T>
static void fill_material(const evpg_rve_desc* d, Material<T>& m) {
    memset(&m, 0, sizeof m);
    for (int p = 0; p < 2; p++) {
        const evpg_phase_desc& s = d->phase[p];
        PhaseK<T>& k = m.ph[p];
        k.crystal = s.crystal;
        k.n_sys = s.n_sys;
        const double kT = d->kT;
        for (int i = 0; i < NS; i++) {
            for (int j = 0; j < NS; j++) {
                k.chi[i][j] = (T)s.chi[i][j];
                k.chi1[i][j] = (T)s.chi1[i][j];
            }
            const double b = s.burgers[i];
            k.k_tpass[i] = (T)(s.c1 * s.shear_g * b * 1.0E-3);
            k.k_tcut[i] = (T)((kT / 0.62415063631) / s.c2 / s.c3 / b / b * 0.1);
            k.k_rhom[i] = (T)(2.0 * kT / s.c1 / s.c2 / s.c3 / s.shear_g / (b * b * b) * 160.2177);
            k.k_gamo[i] = (T)(1E-3 * 1.0E10 * s.c2 * b * exp(-1.0 * s.q_slip));
            k.k_ddip[i] = (T)(sqrt(3.0) * s.shear_g * b / 16.0 / 3.14159265359 / (1 - d->nu));
            k.k_hyd[i] = (T)(s.shear_g * b / 3.14159265359 / (1 - d->nu));
            k.k_d0b[i] = (T)(d->d0 / b);
            k.k_hydr[i] = (T)((s.shear_g * b / 3.14159265359 / (1 - d->nu)) /
                              (sqrt(3.0) * s.shear_g * b / 16.0 / 3.14159265359 / (1 - d->nu)));
            k.k_hexp[i] = (T)(b * b * b * 100 / (1.38 * d->temperature));
            for (int q = 0; q < 5; q++) k.schm_xt[i][q] = (T)s.schm_xt[i][q];
            for (int q = 0; q < 3; q++) {
                k.bn[i][q] = (T)s.bn[i][q];
                k.bb[i][q] = (T)s.bb[i][q];
            }
            k.burgers[i] = (T)b;
        }
        k.tau0 = (T)s.tau0;
        k.shear_g = (T)s.shear_g;
        k.c4 = (T)s.c4;
        k.c5 = (T)s.c5;
        k.c6 = (T)s.c6;
        k.q_bulk = (T)s.q_bulk;
    }
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) {
            m.c066[i][j] = (T)d->c066[i][j];
            m.s066[i][j] = (T)d->s066[i][j];
        }
    for (int i = 0; i < 81; i++) {
        (&m.c0[0][0][0][0])[i] = (T)(&d->c0[0][0][0][0])[i];
        (&m.s0[0][0][0][0])[i] = (T)(&d->s0[0][0][0][0])[i];
    }
    m.dt = (T)d->dt;
    m.kT = (T)d->kT;
    m.temperature = (T)d->temperature;
    m.nu = (T)d->nu;
    m.d0 = (T)d->d0;
    m.elast_bc = d->elast_bc;
}

// ---------------------------------------------------------- field helpers

static void tensor_to_9(const double t[3][3], double* o) {
    sym_to_b6<double>(t, o);
    o[6] = 0.5 * (t[0][1] - t[1][0]);
    o[7] = 0.5 * (t[0][2] - t[2][0]);
    o[8] = 0.5 * (t[1][2] - t[2][1]);
}

static void nine_to_tensor(const double* v, double t[3][3]) {
    b6_to_sym<double>(v, t);
    t[0][1] += v[6]; t[1][0] -= v[6];
    t[0][2] += v[7]; t[2][0] -= v[7];
    t[1][2] += v[8]; t[2][1] -= v[8];
}

struct Alloc {
    Ctx* c;
    template <typename P> cudaError_t get(P** p, size_t n) {
        const size_t b = n * sizeof(P);
        c->bytes += b;
        cudaError_t e = cudaMalloc((void**)p, b ? b : 1);
        if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, b ? b : 1, c->stream);
        return e;
    }
};

static void prof_flush(Ctx& c) {
    Profiler& p = c.prof;
    if (!p.n) return;
    cudaStreamSynchronize(c.stream);
    for (int i = 0; i < p.n; i++) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.recs[i].a, p.recs[i].b) == cudaSuccess) {
            p.ms[p.recs[i].group] += ms;
            p.launches[p.recs[i].group] += 1;
        }
    }
    p.n = 0;
}

void prof_mark(Ctx& c, int group, bool begin) {
    Profiler& p = c.prof;
    if (begin) c.launches++;
    if (!p.on) return;
    if (begin) {
        if (p.n == p.cap) prof_flush(c);
        if (p.n == p.cap) return;
        p.recs[p.n].group = group;
        cudaEventRecord(p.recs[p.n].a, c.stream);
    } else {
        cudaEventRecord(p.recs[p.n].b, c.stream);
        p.n++;
    }
}

static void prof_free(Ctx& c) {
    Profiler& p = c.prof;
    for (int i = 0; i < p.cap; i++) {
        cudaEventDestroy(p.recs[i].a);
        cudaEventDestroy(p.recs[i].b);
    }
    delete[] p.recs;
    p.recs = nullptr;
    p.cap = p.n = 0;
    p.on = false;
}

static void free_ctx(Ctx* c) {
    if (!c) return;
    free_solo(*c);
    prof_free(*c);
    void* ptrs[] = {c->sig64, c->dg64, c->dg_old, c->epsp, c->edot64, c->rho_s, c->rho_m,
                    c->gamdot64, c->gam_acum, c->tranmat, c->schm64, c->fc64, c->sgr64, c->orient,
                    c->phase, c->sig32, c->ddg32, c->b6_32, c->schm32, c->fc32, c->sgr32, c->nrc32, c->spec,
                    c->part_nr, c->part_nr2, c->ticket, c->part_end, c->macro, c->tw64[0], c->tw64[1], c->tw64[2],
                    c->tw32[0], c->tw32[1], c->tw32[2], c->rho_g, c->gproj, c->gbm};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (c->macro_host) cudaFreeHost(c->macro_host);
    if (c->ctl_host) cudaFreeHost(c->ctl_host);
    if (c->dl_dev) cudaFree(c->dl_dev);
    if (c->dl_host) cudaFreeHost(c->dl_host);
    for (int i = 0; i < 2; i++)
        if (c->dl_ev[i]) cudaEventDestroy(c->dl_ev[i]);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c->ks;
    delete c;
}

void set_kernel_attributes() {
    static std::mutex mu;
    static unsigned long long done_mask = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && (done_mask >> dev) & 1ULL) return;
    spectral_attributes();
    solver_attributes();
    if (dev >= 0 && dev < 64) done_mask |= 1ULL << dev;
}

void build_sets(Ctx& c) {
    build_spectral_sets(c);
    build_solver_sets(c);
}

}  // namespace evpg

using namespace evpg;

extern "C" {

const char* evpg_version(void) { return "evpg 0.1 (sm_103a)"; }

const char* evpg_last_error(void) { return g_err; }

const char* evpg_status_string(int st) {
    switch (st) {
        case EVPG_OK: return "ok";
        case EVPG_ERR_ARG: return "invalid argument";
        case EVPG_ERR_CUDA: return "CUDA error";
        case EVPG_ERR_NOMEM: return "out of memory";
        case EVPG_ERR_NAN: return "NaN in the flow rule";
        case EVPG_ERR_SINGULAR: return "singular 6x6 system";
        case EVPG_ERR_LINESEARCH: return "line search found no descent direction";
        case EVPG_ERR_ITERMAX: return "equilibrium loop reached IterMax";
        case EVPG_ERR_IO: return "input file error";
        case EVPG_ERR_NO_DEVICE: return "no CUDA device";
        case EVPG_ERR_TIMEOUT: return "device-side wait exceeded its bound";
        default: return "unknown status";
    }
}

// Host-side GND constants: per phase the projection tables and sense vectors
// of the GP_* row (init.c:198-203, 1119-1140), and per voxel the same-grain
// bits of Gradient_ExchangeGrainID (constitutive.c:731-879) on one rank with
// periodic neighbours: bit 0/1 x+/x-, 2/3 y+/y-, 4 z+, 5 the reference's
// "z-" check, which compares with the y- neighbour (GB_checkZ[pIDX][1]).
static void gnd_tables(const evpg_rve_desc* d, std::vector<double>& gp, std::vector<uint8_t>& m) {
    gp.assign(2 * (size_t)GP_STRIDE, 0.0);
    for (int p = 0; p < 2; p++) {
        const evpg_phase_desc& P = d->phase[p];
        double* row = gp.data() + (size_t)p * GP_STRIDE;
        for (int i = 0; i < P.n_sys; i++) {
            const double *ni = P.bn[i], *bi = P.bb[i];
            row[GP_BP + 3 * i + 0] = bi[1] * ni[2] - bi[2] * ni[1];
            row[GP_BP + 3 * i + 1] = bi[2] * ni[0] - bi[0] * ni[2];
            row[GP_BP + 3 * i + 2] = bi[0] * ni[1] - bi[1] * ni[0];
            for (int j = 0; j < P.n_sys; j++) {
                const double *nj = P.bn[j], *bj = P.bb[j];
                const double sv[3] = {nj[1] * bj[2] - nj[2] * bj[1], nj[2] * bj[0] - nj[0] * bj[2],
                                      nj[0] * bj[1] - nj[1] * bj[0]};
                const double cs = fabs(ni[0] * sv[0] + ni[1] * sv[1] + ni[2] * sv[2]);
                const double c1 = fabs(ni[0] * bj[0] + ni[1] * bj[1] + ni[2] * bj[2]);
                row[GP_COS1 + i * NS + j] = c1;
                row[GP_SIN1 + i * NS + j] = fabs(sqrt(fabs(1.0 - c1 * c1)));
                row[GP_COS2 + i * NS + j] = cs;
                row[GP_SIN2 + i * NS + j] = fabs(sqrt(fabs(1.0 - cs * cs)));
            }
        }
    }
    const int n0 = d->n[0], n1 = d->n[1], n2 = d->n[2];
    const int32_t* g = d->voxel_grain;
    m.assign((size_t)n0 * n1 * n2, 0);
    for (int x = 0; x < n0; x++)
        for (int y = 0; y < n1; y++)
            for (int z = 0; z < n2; z++) {
                const int xp = (x + 1) % n0, xm = (x + n0 - 1) % n0, yp = (y + 1) % n1,
                          ym = (y + n1 - 1) % n1, zp = (z + 1) % n2;
                const size_t v = ((size_t)x * n1 + y) * n2 + z;
                const int gv = g[v];
                auto at = [&](int a, int b, int c) { return g[((size_t)a * n1 + b) * n2 + c]; };
                m[v] = (uint8_t)((gv == at(xp, y, z)) | (gv == at(xm, y, z)) << 1 | (gv == at(x, yp, z)) << 2 |
                                 (gv == at(x, ym, z)) << 3 | (gv == at(x, y, zp)) << 4 |
                                 (gv == at(x, ym, z)) << 5);
            }
}

int evpg_create(const evpg_rve_desc* d, void** out) {
    if (!d || !out) return fail(EVPG_ERR_ARG, "null argument");
    *out = nullptr;
    for (int i = 0; i < 3; i++)
        if (d->n[i] < 1 || d->n[i] > 1024) return fail(EVPG_ERR_ARG, "grid size %d out of range", d->n[i]);
    const long long NN = (long long)d->n[0] * d->n[1] * d->n[2];
    if (NN > (1LL << 30)) return fail(EVPG_ERR_ARG, "grid too large");
    if (d->precision != EVPG_FP64 && d->precision != EVPG_FP32_BULK)
        return fail(EVPG_ERR_ARG, "precision %d", d->precision);
    if (d->nr_mode != EVPG_NR_PLAIN && d->nr_mode != EVPG_NR_LINESEARCH)
        return fail(EVPG_ERR_ARG, "nr_mode %d", d->nr_mode);
    if (!d->voxel_orient || !d->voxel_phase || !d->tranmat || !d->sig0 || !d->rho_s0 ||
        (d->n_orient > 0 && (!d->c_gr || !d->s_gr)))
        return fail(EVPG_ERR_ARG, "missing RVE arrays");
    for (int p = 0; p < 2; p++)
        if (d->phase[p].n_sys < 0 || d->phase[p].n_sys > EVPG_NSYS)
            return fail(EVPG_ERR_ARG, "n_sys %d", d->phase[p].n_sys);
    if (d->gnd && (!d->voxel_grain || !(d->l0 > 0.0)))
        return fail(EVPG_ERR_ARG, "GND densities need voxel_grain and L0 > 0");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(EVPG_ERR_NO_DEVICE, "no CUDA device");
    const int N = (int)NN;
    for (int v = 0; v < N; v++) {
        const int ph = d->voxel_phase[v];
        if (ph < 1 || ph > 2) return fail(EVPG_ERR_ARG, "voxel %d: phase %d", v, ph);
        if (d->phase[ph - 1].crystal && (d->voxel_orient[v] < 0 || d->voxel_orient[v] >= d->n_orient))
            return fail(EVPG_ERR_ARG, "voxel %d: orientation %d", v, d->voxel_orient[v]);
    }
    Ctx* c = new Ctx();
    memset((void*)c, 0, sizeof(Ctx));
    c->g.n0 = d->n[0]; c->g.n1 = d->n[1]; c->g.n2 = d->n[2];
    c->g.nh = d->n[2] / 2 + 1;
    c->g.N = N;
    c->g.Nh = (long long)d->n[0] * d->n[1] * c->g.nh;
    c->precision = d->precision;
    c->nr_mode = d->nr_mode;
    c->n_orient = d->n_orient;
    c->nr_itmax = 500;
    c->nr_tol64 = 1E-10;
    c->nr_tol32 = 1E-5;  // FP32: same iteration counts and errors as 2e-6 at 64^3 and 128^3, 6 % faster
    c->delta_tau_drx = d->delta_tau_drx;
    c->tau_drx = d->tau_drx;
    memcpy(c->udot_a, d->udot_a, sizeof c->udot_a);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return fail(EVPG_ERR_CUDA, "stream creation failed");
    }
    c->own_stream = true;
    for (int a = 0; a < 3; a++) make_plan(d->n[a], c->pl[a]);
    fill_material<double>(d, c->m64);
    fill_material<float>(d, c->m32);
    memcpy(c->cfg.s0, d->s0, sizeof c->cfg.s0);
    memcpy(c->cfg.scauchy, d->scauchy, sizeof c->cfg.scauchy);
    for (int i = 0; i < 6; i++) {
        c->cfg.vflag[i] = d->velgrad_bc_flag[i];
        c->cfg.sflag[i] = d->stress_bc_flag[i];
    }
    c->cfg.wgt = 1. / N;
    c->cfg.wgt_ph1 = d->wgt_ph1;
    c->cfg.err_tol = d->err_tol;
    c->cfg.iter_max = d->iter_max;
    c->nb_nr = (N + NR_BLOCK - 1) / NR_BLOCK;
    c->nb_end = (N + END_BLOCK - 1) / END_BLOCK;

    Alloc A{c};
    const size_t n = (size_t)N;
    const bool f32 = c->precision == EVPG_FP32_BULK;
    cudaError_t e = cudaSuccess;
#define AL(p, cnt) \
    if (e == cudaSuccess) e = A.get(&(p), (cnt))
    AL(c->sig64, 6 * n); AL(c->dg64, 9 * n); AL(c->dg_old, 9 * n); AL(c->epsp, 6 * n);
    AL(c->edot64, 5 * n); AL(c->rho_s, 12 * n); AL(c->rho_m, 12 * n); AL(c->gamdot64, 12 * n);
    AL(c->gam_acum, 12 * n); AL(c->tranmat, 9 * n); AL(c->schm64, 60 * n); AL(c->fc64, 48 * n);
    AL(c->sgr64, SGR_STRIDE * (size_t)(d->n_orient > 0 ? d->n_orient : 1));
    AL(c->orient, n); AL(c->phase, n);
    if (f32) {
        AL(c->sig32, 6 * n); AL(c->ddg32, 9 * n); AL(c->b6_32, 6 * n); AL(c->schm32, 60 * n);
        AL(c->fc32, 48 * n); AL(c->sgr32, SGR_STRIDE * (size_t)(d->n_orient > 0 ? d->n_orient : 1));
        AL(c->nrc32, (size_t)c->nb_nr * NRC_BLOCK_FLOATS);
        // nine spectrum components, the sum of the deferred antisymmetric ones
        // and their pending values of the current iteration
        float2* sp = nullptr;
        AL(sp, 15 * (size_t)c->g.Nh);
        c->spec = sp;
    } else {
        double2* sp = nullptr;
        AL(sp, 9 * (size_t)c->g.Nh);
        c->spec = sp;
    }
    if (d->gnd) {
        AL(c->rho_g, 24 * n); AL(c->gproj, 2 * (size_t)GP_STRIDE); AL(c->gbm, n);
        c->l0 = d->l0;
    }
    AL(c->part_nr, (size_t)c->nb_nr * (NR_BLOCK / 32) * NPART_NR);
    AL(c->part_nr2, (size_t)MACRO_BLOCKS * NPART_NR);
    AL(c->ticket, 1);
    AL(c->part_end, (size_t)c->nb_end * NPART_END);
    AL(c->macro, 1);
    for (int a = 0; a < 3; a++) {
        AL(c->tw64[a], (size_t)d->n[a]);
        AL(c->tw32[a], (size_t)d->n[a]);
    }
#undef AL
    if (e == cudaSuccess) e = cudaMallocHost((void**)&c->macro_host, sizeof(Macro));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&c->ctl_host, sizeof(IncrCtl));
    if (e != cudaSuccess) {
        free_ctx(c);
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? EVPG_ERR_NOMEM : EVPG_ERR_CUDA,
                    "allocation: %s", cudaGetErrorString(e));
    }
    memset(c->macro_host, 0, sizeof(Macro));
    memset(c->ctl_host, 0, sizeof(IncrCtl));

    // host-side layout changes: AoS tensors -> SoA planes in the B basis
    std::vector<double> h(60 * n);
    auto put = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
        cudaError_t r = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
        if (r == cudaSuccess) r = cudaStreamSynchronize(c->stream);
        return r;
    };
    for (size_t v = 0; v < n; v++) {
        double t[3][3], o[6];
        memcpy(t, d->sig0 + 9 * v, sizeof t);
        sym_to_b6<double>(t, o);
        for (int q = 0; q < 6; q++) h[q * n + v] = o[q];
    }
    e = put(c->sig64, h.data(), 6 * n * sizeof(double));
    if (e == cudaSuccess && f32) {
        std::vector<float> hf(6 * n);
        for (size_t i = 0; i < 6 * n; i++) hf[i] = (float)h[i];
        e = put(c->sig32, hf.data(), 6 * n * sizeof(float));
    }
    for (size_t v = 0; v < n; v++)
        for (int q = 0; q < 9; q++) h[q * n + v] = d->tranmat[9 * v + q];
    if (e == cudaSuccess) e = put(c->tranmat, h.data(), 9 * n * sizeof(double));
    for (size_t v = 0; v < n; v++)
        for (int q = 0; q < 12; q++) h[q * n + v] = d->rho_s0[12 * v + q];
    if (e == cudaSuccess) e = put(c->rho_s, h.data(), 12 * n * sizeof(double));
    if (e == cudaSuccess) e = put(c->orient, d->voxel_orient, n * sizeof(int32_t));
    if (e == cudaSuccess) e = put(c->phase, d->voxel_phase, n * sizeof(int32_t));
    if (e == cudaSuccess && d->n_orient > 0) {
        // per orientation: S_gr (36) and the constant part of the NR matrix,
        // packed upper triangle of S066 + (S_gr + S_gr^T)/2 (21)
        std::vector<double> t(SGR_STRIDE * (size_t)d->n_orient, 0.0);
        for (int o = 0; o < d->n_orient; o++) {
            const double* sg = d->s_gr + 36 * (size_t)o;
            double* row = t.data() + SGR_STRIDE * (size_t)o;
            memcpy(row, sg, 36 * sizeof(double));
            int k = 0;
            for (int i = 0; i < 6; i++)
                for (int j = i; j < 6; j++) row[36 + k++] = d->s066[i][j] + 0.5 * (sg[i * 6 + j] + sg[j * 6 + i]);
        }
        e = put(c->sgr64, t.data(), t.size() * sizeof(double));
        if (e == cudaSuccess && f32) {
            // FP32 rows: packed upper triangle of (S_gr + S_gr^T)/2 only (21);
            // the NR adds S066 from its constant bank. S_gr is symmetric up to
            // the rounding of its inversion, far below FP32 resolution.
            std::vector<float> hf(t.size(), 0.0f);
            for (int o = 0; o < d->n_orient; o++) {
                const double* sg = d->s_gr + 36 * (size_t)o;
                float* row = hf.data() + SGR_STRIDE * (size_t)o;
                int k = 0;
                for (int i = 0; i < 6; i++)
                    for (int j = i; j < 6; j++) row[k++] = (float)(0.5 * (sg[i * 6 + j] + sg[j * 6 + i]));
            }
            e = put(c->sgr32, hf.data(), hf.size() * sizeof(float));
        }
    }
    if (e == cudaSuccess && d->gnd) {
        std::vector<double> gp;
        std::vector<uint8_t> m;
        gnd_tables(d, gp, m);
        e = put(c->gproj, gp.data(), gp.size() * sizeof(double));
        if (e == cudaSuccess) e = put(c->gbm, m.data(), m.size());
    }
    for (int a = 0; a < 3 && e == cudaSuccess; a++) {
        const int na = d->n[a];
        std::vector<double2> t64(na);
        std::vector<float2> t32(na);
        for (int t = 0; t < na; t++) {
            double cc, ss;
            unit_root(t, na, &cc, &ss);
            t64[t] = make_double2(cc, ss);
            t32[t] = make_float2((float)cc, (float)ss);
        }
        e = put(c->tw64[a], t64.data(), na * sizeof(double2));
        if (e == cudaSuccess) e = put(c->tw32[a], t32.data(), na * sizeof(float2));
    }
    // an idle context: no increment requested, loop finished
    if (e == cudaSuccess) {
        c->macro_host->done = 1;
        c->macro_host->ctl.phase = PH_IDLE;
        e = put(c->macro, c->macro_host, sizeof(Macro));
    }
    if (e != cudaSuccess) {
        free_ctx(c);
        return fail(EVPG_ERR_CUDA, "upload: %s", cudaGetErrorString(e));
    }
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev);
    }
    set_kernel_attributes();
    c->sched_fused = -1;
    c->sched_xpass = -1;
    for (int i = 0; i < 2 && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&c->dl_ev[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        free_ctx(c);
        return fail(EVPG_ERR_CUDA, "event creation: %s", cudaGetErrorString(e));
    }
    c->ks = new KernelSets();
    memset((void*)c->ks, 0, sizeof(KernelSets));
    build_sets(*c);
    *out = c;
    return EVPG_OK;
}

int evpg_destroy(void* ctx) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return EVPG_OK;
    cudaStreamSynchronize(c->stream);
    free_ctx(c);
    return EVPG_OK;
}

int evpg_set_stream(void* ctx, void* s) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(EVPG_ERR_ARG, "null context");
    CK(cudaStreamSynchronize(c->stream));
    if (c->own_stream) cudaStreamDestroy(c->stream);
    if (s) {
        c->stream = (cudaStream_t)s;
        c->own_stream = false;
    } else {
        CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    return EVPG_OK;
}

int evpg_device_bytes(void* ctx, int64_t* bytes) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !bytes) return fail(EVPG_ERR_ARG, "null argument");
    *bytes = (int64_t)c->bytes;
    return EVPG_OK;
}

int evpg_profile(void* ctx, int32_t enable) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(EVPG_ERR_ARG, "null context");
    if (enable && !c->prof.recs) {
        c->prof.cap = 4096;
        c->prof.recs = new Profiler::Rec[c->prof.cap];
        for (int i = 0; i < c->prof.cap; i++) {
            CK(cudaEventCreate(&c->prof.recs[i].a));
            CK(cudaEventCreate(&c->prof.recs[i].b));
        }
    }
    prof_flush(*c);
    for (int g = 0; g < PG_COUNT; g++) {
        c->prof.ms[g] = 0.0;
        c->prof.launches[g] = 0;
    }
    c->prof.on = enable != 0;
    return EVPG_OK;
}

int evpg_launch_count(void* ctx, int64_t* n) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !n) return fail(EVPG_ERR_ARG, "null argument");
    *n = c->launches;
    return EVPG_OK;
}

int evpg_profile_read(void* ctx, double* ms, int64_t* launches, int32_t n) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !ms || !launches) return fail(EVPG_ERR_ARG, "null argument");
    prof_flush(*c);
    for (int g = 0; g < n && g < PG_COUNT; g++) {
        ms[g] = c->prof.ms[g];
        launches[g] = c->prof.launches[g];
    }
    return EVPG_OK;
}

int evpg_synchronize(void* ctx) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(EVPG_ERR_ARG, "null context");
    CK(cudaStreamSynchronize(c->stream));
    return EVPG_OK;
}

}  // extern "C"

namespace evpg {

__global__ void k_set_evm(Macro* m, double e_vm) {
    m->e_vm = e_vm;
    m->ctl.e_vm = e_vm;
}

__global__ void k_set_tail(Macro* m, int t) { m->ctl.tail = t; }

// Field packing for downloads: SoA planes (B basis) -> voxel-major records
// in the host layout of evpg_download, for voxels [v0, v0 + nv).
enum PackKind { PK_TENSOR6 = 0, PK_SIG6 = 1, PK_TENSOR9 = 2, PK_EDOT5 = 3, PK_COPY = 4 };

__global__ void k_pack(const double* __restrict__ src, size_t N, int planes, int kind, size_t v0, int nv,
                       double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const size_t v = v0 + (size_t)i;
    double q[12];
#pragma unroll
    for (int p = 0; p < 12; p++) q[p] = p < planes ? src[(size_t)p * N + v] : 0.0;
    if (kind == PK_COPY) {
        for (int p = 0; p < planes; p++) out[(size_t)i * planes + p] = q[p];
        return;
    }
    double t[3][3];
    if (kind == PK_TENSOR9) {
        b6_to_sym<double>(q, t);
        t[0][1] += q[6]; t[1][0] -= q[6];
        t[0][2] += q[7]; t[2][0] -= q[7];
        t[1][2] += q[8]; t[2][1] -= q[8];
    } else {
        if (kind == PK_EDOT5) q[5] = 0.0;
        b6_to_sym<double>(q, t);
    }
    if (kind == PK_SIG6) {
        double* o = out + (size_t)i * 6;
        o[0] = t[0][0]; o[1] = t[1][1]; o[2] = t[2][2];
        o[3] = t[1][2]; o[4] = t[0][2]; o[5] = t[0][1];
    } else {
        double* o = out + (size_t)i * 9;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) o[3 * a + b] = t[a][b];
    }
}

static int read_macro(Ctx* c) {
    CK(cudaMemcpyAsync(c->macro_host, c->macro, sizeof(Macro), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return EVPG_OK;
}

static void fill_iter_out(const Macro& m, evpg_iter_out* o) {
    o->err_e = m.err_e;
    o->err_s = m.err_s;
    o->err_e_sum = m.err_e_sum;
    o->err_s_sum = m.err_s_sum;
    memcpy(o->sig_avg, m.sig_avg, sizeof o->sig_avg);
    memcpy(o->sig_avg_ph1, m.sig_avg1, sizeof o->sig_avg_ph1);
    memcpy(o->ddisgrad, m.dE, sizeof o->ddisgrad);
    memcpy(o->ddisgrad_acum, m.dE_acum, sizeof o->ddisgrad_acum);
    o->s_vm = m.s_vm;
    o->s_vm1 = m.s_vm1;
    o->iter = m.iter;
    o->converged = m.converged;
}

static int launch_iteration(Ctx* c) {
    CK(launch_spectral(*c, GATE_RUNNING));
    CK(launch_nr(*c, 0, GATE_RUNNING));
    CK(launch_macro(*c));
    return EVPG_OK;
}

// Controls of one increment into the context's pinned staging area.
static void stage_ctl(Ctx* c, const double udot_dt[3][3], int creep, const double dgavg[3][3],
                      double time_tot, double e_vm, int tail) {
    IncrCtl& k = *c->ctl_host;
    double u9[9], g9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    tensor_to_9(udot_dt, u9);
    if (creep) tensor_to_9(dgavg, g9);
    memcpy(k.udot9, u9, sizeof u9);
    memcpy(k.dgavg9, g9, sizeof g9);
    // DeltaTau_DRX*exp((t_last-TimeTot)/TimeStep/tau_DRX), t_last = -1E3*tau_DRX*TimeStep
    const double dt = c->m64.dt;
    const double t_last = -1E3 * c->tau_drx * dt;
    k.drx = c->delta_tau_drx * exp((t_last - time_tot) / dt / c->tau_drx);
    k.e_vm = e_vm;
    k.err0 = 2. * c->cfg.err_tol;
    k.creep = creep ? 1 : 0;
    k.tail = tail & (EVPG_TAIL_REORIENT | EVPG_TAIL_GND_GRADIENT);
    k.phase = PH_BEGIN;
    k.pad = 0;
}

}  // namespace evpg

extern "C" {

int evpg_increment_begin(void* ctx, const double udot_dt[3][3], int32_t creep,
                         const double dgavg[3][3], double time_tot) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !udot_dt) return fail(EVPG_ERR_ARG, "null argument");
    if (creep && !dgavg) return fail(EVPG_ERR_ARG, "creep needs disgrad_avg_actual");
    // the staging area may still feed an earlier copy
    CK(cudaStreamSynchronize(c->stream));
    stage_ctl(c, udot_dt, creep, dgavg, time_tot, 0.0, 0);
    CK(cudaMemcpyAsync(c->macro, c->ctl_host, sizeof(IncrCtl), cudaMemcpyHostToDevice, c->stream));
    CK(launch_macro_begin(*c, GATE_BEGIN));
    CK(launch_begin(*c, GATE_BEGIN));
    CK(launch_phase(*c, PH_BEGIN, PH_RUNNING));
    return EVPG_OK;
}

int evpg_equilibrium_iteration(void* ctx, double e_vm, evpg_iter_out* out) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(EVPG_ERR_ARG, "null context");
    k_set_evm<<<1, 1, 0, c->stream>>>(c->macro, e_vm);
    c->launches++;
    CK(cudaGetLastError());
    int st = launch_iteration(c);
    if (st) return st;
    st = read_macro(c);
    if (st) return st;
    if (out) fill_iter_out(*c->macro_host, out);
    if (c->macro_host->status) return fail(c->macro_host->status, "%s", evpg_status_string(c->macro_host->status));
    return EVPG_OK;
}

int evpg_equilibrium_solve(void* ctx, double e_vm, evpg_iter_out* out) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(EVPG_ERR_ARG, "null context");
    k_set_evm<<<1, 1, 0, c->stream>>>(c->macro, e_vm);
    c->launches++;
    CK(cudaGetLastError());
    int batch = c->prof.on ? 1 : 2;
    for (;;) {
        for (int b = 0; b < batch; b++) {
            const int st = launch_iteration(c);
            if (st) return st;
        }
        const int st = read_macro(c);
        if (st) return st;
        if (c->macro_host->done) break;
        if (!c->prof.on && batch < 16) batch *= 2;
    }
    if (out) fill_iter_out(*c->macro_host, out);
    if (c->macro_host->status) return fail(c->macro_host->status, "%s", evpg_status_string(c->macro_host->status));
    return EVPG_OK;
}

int evpg_increment_end(void* ctx, int32_t tail, evpg_incr_out* out) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(EVPG_ERR_ARG, "null context");
    k_set_tail<<<1, 1, 0, c->stream>>>(c->macro, tail & (EVPG_TAIL_REORIENT | EVPG_TAIL_GND_GRADIENT));
    c->launches++;
    if (c->precision == EVPG_FP32_BULK) {
        CK(launch_fold(*c, GATE_ALWAYS));
        CK(launch_nr(*c, 1, GATE_ALWAYS));
    }
    CK(launch_end(*c, GATE_ALWAYS));
    CK(launch_phase(*c, PH_RUNNING, PH_ENDED));
    int st = read_macro(c);
    if (st) return st;
    const Macro& m = *c->macro_host;
    if (out) {
        double e6[6], d6[6];
        memcpy(e6, m.eps_avg6, sizeof e6);
        memcpy(d6, m.edot_avg6, sizeof d6);
        b6_to_sym<double>(e6, out->eps_avg);
        b6_to_sym<double>(d6, out->edot_avg);
        memcpy(out->rho_avg, m.rho_avg, sizeof out->rho_avg);
        out->nr_iterations = m.nr_iters;
    }
    if (m.status) return fail(m.status, "%s", evpg_status_string(m.status));
    return EVPG_OK;
}

int evpg_set_load(void* ctx, const int32_t velgrad_bc_flag[6], const int32_t stress_bc_flag[6],
                  const double scauchy[3][3], const double udot_a[3][3]) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !velgrad_bc_flag || !stress_bc_flag || !scauchy || !udot_a)
        return fail(EVPG_ERR_ARG, "null argument");
    for (int i = 0; i < 6; i++)
        if (velgrad_bc_flag[i] * stress_bc_flag[i] != 0 || velgrad_bc_flag[i] + stress_bc_flag[i] != 1)
            return fail(EVPG_ERR_ARG, "component %d: exactly one of velocity gradient and stress is prescribed", i);
    CK(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < 6; i++) {
        c->cfg.vflag[i] = velgrad_bc_flag[i];
        c->cfg.sflag[i] = stress_bc_flag[i];
    }
    memcpy(c->cfg.scauchy, scauchy, sizeof c->cfg.scauchy);
    memcpy(c->udot_a, udot_a, sizeof c->udot_a);
    build_sets(*c);
    c->version++;
    return EVPG_OK;
}

int evpg_tune(void* ctx, int32_t force, double* gain) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(EVPG_ERR_ARG, "null context");
    const int st = tune_spectral(*c, force ? 1 : 0, gain);
    if (st == 3) return fail(EVPG_ERR_NOMEM, "autotuner scratch allocation failed");
    if (st) return fail(EVPG_ERR_CUDA, "autotuner launch failed");
    return EVPG_OK;
}

int evpg_set_nr_tolerance(void* ctx, double tol, int32_t itmax) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !(tol > 0.0) || itmax < 1) return fail(EVPG_ERR_ARG, "bad argument");
    CK(cudaStreamSynchronize(c->stream));
    if (c->precision == EVPG_FP32_BULK) c->nr_tol32 = tol;
    else c->nr_tol64 = tol;
    c->nr_itmax = itmax;
    build_sets(*c);
    c->version++;
    return EVPG_OK;
}

int evpg_set_fused(void* ctx, int32_t mode) {
    Ctx* c = (Ctx*)ctx;
    if (!c || mode < -1 || mode > 1) return fail(EVPG_ERR_ARG, "bad argument");
    CK(cudaStreamSynchronize(c->stream));
    c->sched_fused = mode;
    build_sets(*c);
    c->version++;
    return EVPG_OK;
}

int evpg_set_xpass(void* ctx, int32_t mode) {
    Ctx* c = (Ctx*)ctx;
    if (!c || mode < -1 || mode > 1) return fail(EVPG_ERR_ARG, "bad argument");
    CK(cudaStreamSynchronize(c->stream));
    c->sched_xpass = mode;
    build_sets(*c);
    c->version++;
    return EVPG_OK;
}

int evpg_set_radix(void* ctx, int32_t axis, const int32_t* radix, int32_t nstages) {
    Ctx* c = (Ctx*)ctx;
    if (!c || axis < 0 || axis > 2 || !radix || nstages < 1 || nstages > 12)
        return fail(EVPG_ERR_ARG, "bad argument");
    long long prod = 1;
    for (int s = 0; s < nstages; s++) {
        const int r = radix[s];
        // radix 16 runs in the FP32 x transforms only
        if (r < 2 || (r == 16 && (c->precision == EVPG_FP64 || axis != 0)))
            return fail(EVPG_ERR_ARG, "radix %d on axis %d", r, axis);
        prod *= r;
    }
    const int n = axis == 0 ? c->g.n0 : axis == 1 ? c->g.n1 : c->g.n2;
    if (prod != n) return fail(EVPG_ERR_ARG, "radices do not multiply to %d", n);
    CK(cudaStreamSynchronize(c->stream));
    FftPlan& p = c->pl[axis];
    memset(&p, 0, sizeof p);
    p.n = n;
    p.nf = nstages;
    int ns = 1;
    for (int s = 0; s < nstages; s++) {
        p.radix[s] = radix[s];
        p.ns[s] = ns;
        ns *= radix[s];
    }
    plan_divisors(p);
    build_sets(*c);
    c->version++;
    return EVPG_OK;
}

int evpg_get_schedule(void* ctx, int32_t pencils[3], int32_t radix[3][12], int32_t nstages[3]) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(EVPG_ERR_ARG, "null context");
    const int prec = c->precision;
    const int epl = prec ? c->ks->s32.epl : c->ks->s64.epl;
    // fused z+y plane kernels: the z and y entries are 0 (one x plane per CTA)
    const int P[3] = {epl ? 0 : (prec ? c->ks->s32.z.P : c->ks->s64.z.P),
                      epl ? 0 : (prec ? c->ks->s32.yf.P : c->ks->s64.yf.P),
                      prec ? c->ks->s32.x.P : c->ks->s64.x.P};
    for (int a = 0; a < 3; a++) {
        if (pencils) pencils[a] = P[a];
        if (nstages) nstages[a] = c->pl[a].nf;
        if (radix)
            for (int s = 0; s < 12; s++) radix[a][s] = s < c->pl[a].nf ? c->pl[a].radix[s] : 0;
    }
    return EVPG_OK;
}

int evpg_get_variant(void* ctx, int32_t variant[2]) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !variant) return fail(EVPG_ERR_ARG, "bad argument");
    variant[0] = c->precision ? c->ks->s32.epl : c->ks->s64.epl;
    variant[1] = c->precision ? c->ks->s32.xw : c->ks->s64.xw;
    return EVPG_OK;
}

int evpg_estimate_bytes(const int32_t n[3], int32_t precision, int32_t n_orient, int64_t* bytes) {
    if (!n || !bytes || n[0] < 1 || n[1] < 1 || n[2] < 1) return fail(EVPG_ERR_ARG, "bad argument");
    const long long N = (long long)n[0] * n[1] * n[2];
    const long long Nh = (long long)n[0] * n[1] * (n[2] / 2 + 1);
    const long long no = n_orient > 0 ? n_orient : 1;
    const long long nb_nr = (N + NR_BLOCK - 1) / NR_BLOCK, nb_end = (N + END_BLOCK - 1) / END_BLOCK;
    long long b = 8 * N * (6 + 9 + 9 + 6 + 5 + 12 + 12 + 12 + 12 + 9 + 60 + 48) + 8 * SGR_STRIDE * no + 4 * 2 * N;
    if (precision == EVPG_FP32_BULK)
        b += 4 * N * (6 + 9 + 6 + 60 + 48) + 4 * SGR_STRIDE * no + 8 * 15 * Nh + 4 * nb_nr * NRC_BLOCK_FLOATS;
    else b += 16 * 9 * Nh;
    b += 8 * nb_nr * (NR_BLOCK / 32) * NPART_NR + 8 * MACRO_BLOCKS * NPART_NR + 4 + 8 * nb_end * NPART_END;
    b += (long long)sizeof(Macro) + 24LL * (n[0] + n[1] + n[2]);
    b += 2LL * (long long)dl_chunk_doubles((size_t)N) * 8;  // download packing buffers
    *bytes = b;
    return EVPG_OK;
}

int evpg_download(void* ctx, int32_t field, double* host, size_t count) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !host) return fail(EVPG_ERR_ARG, "null argument");
    const size_t n = (size_t)c->g.N;
    const double* src = nullptr;
    int planes = 0, kind = PK_COPY, outw = 12;
    switch (field) {
        case EVPG_F_SIG: src = c->sig64; planes = 6; kind = PK_TENSOR6; outw = 9; break;
        case EVPG_F_SIG6: src = c->sig64; planes = 6; kind = PK_SIG6; outw = 6; break;
        case EVPG_F_DISGRAD: src = c->dg64; planes = 9; kind = PK_TENSOR9; outw = 9; break;
        case EVPG_F_EPS: src = c->epsp; planes = 6; kind = PK_TENSOR6; outw = 9; break;
        case EVPG_F_EDOT: src = c->edot64; planes = 5; kind = PK_EDOT5; outw = 9; break;
        case EVPG_F_TRANMAT: src = c->tranmat; planes = 9; kind = PK_COPY; outw = 9; break;
        case EVPG_F_RHO_S: src = c->rho_s; planes = 12; break;
        case EVPG_F_RHO_M: src = c->rho_m; planes = 12; break;
        case EVPG_F_GAMDOT: src = c->gamdot64; planes = 12; break;
        case EVPG_F_GAM_ACUM: src = c->gam_acum; planes = 12; break;
        case EVPG_F_VELGRAD: src = c->dg_old; planes = 9; kind = PK_TENSOR9; outw = 9; break;
        case EVPG_F_RHO_G1: src = c->rho_g; planes = 12; break;
        case EVPG_F_RHO_G2: src = c->rho_g ? c->rho_g + 12 * n : nullptr; planes = 12; break;
        default: return fail(EVPG_ERR_ARG, "unknown field %d", field);
    }
    if (!src) return fail(EVPG_ERR_ARG, "field %d: GND densities are off for this context", field);
    if (count < (size_t)outw * n) return fail(EVPG_ERR_ARG, "buffer too small");
    // packed on the device in chunks, copied through a pinned staging buffer
    // (or straight into the caller's buffer when it is pinned)
    const size_t cap = dl_chunk_doubles(n);
    const size_t chunk = cap / (size_t)outw;
    if (!c->dl_dev) {
        CK(cudaMalloc((void**)&c->dl_dev, 2 * cap * sizeof(double)));
        c->bytes += 2 * cap * sizeof(double);
        CK(cudaMallocHost((void**)&c->dl_host, 2 * cap * sizeof(double)));
    }
    cudaPointerAttributes pa;
    bool pinned = cudaPointerGetAttributes(&pa, host) == cudaSuccess && pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    int k = 0;
    size_t done_v = 0, pend_v0 = 0, pend_nv = 0;
    for (size_t v0 = 0; v0 < n; v0 += chunk, k ^= 1) {
        const size_t nv = (n - v0 < chunk) ? n - v0 : chunk;
        double* dbuf = c->dl_dev + (size_t)k * cap;
        k_pack<<<(unsigned)((nv + 255) / 256), 256, 0, c->stream>>>(src, n, planes, kind, v0, (int)nv, dbuf);
        c->launches++;
        double* dst = pinned ? host + v0 * outw : c->dl_host + (size_t)k * cap;
        CK(cudaMemcpyAsync(dst, dbuf, nv * outw * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        if (!pinned) {
            // finish the previous chunk on the host while this one copies
            if (pend_nv) {
                CK(cudaEventSynchronize(c->dl_ev[k ^ 1]));
                memcpy(host + pend_v0 * outw, c->dl_host + (size_t)(k ^ 1) * cap, pend_nv * outw * sizeof(double));
            }
            CK(cudaEventRecord(c->dl_ev[k], c->stream));
            pend_v0 = v0;
            pend_nv = nv;
        }
        done_v += nv;
    }
    CK(cudaStreamSynchronize(c->stream));
    if (!pinned && pend_nv)
        memcpy(host + pend_v0 * outw, c->dl_host + (size_t)(k ^ 1) * cap, pend_nv * outw * sizeof(double));
    (void)done_v;
    return EVPG_OK;
}

int evpg_upload(void* ctx, int32_t field, const double* host, size_t count) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !host) return fail(EVPG_ERR_ARG, "null argument");
    const size_t n = (size_t)c->g.N;
    double* dst = nullptr;
    int planes = 0;
    switch (field) {
        case EVPG_F_SIG: dst = c->sig64; planes = 6; break;
        case EVPG_F_DISGRAD: dst = c->dg64; planes = 9; break;
        case EVPG_F_EPS: dst = c->epsp; planes = 6; break;
        case EVPG_F_TRANMAT: dst = c->tranmat; planes = 9; break;
        case EVPG_F_RHO_S: dst = c->rho_s; planes = 12; break;
        case EVPG_F_RHO_M: dst = c->rho_m; planes = 12; break;
        case EVPG_F_GAM_ACUM: dst = c->gam_acum; planes = 12; break;
        default: return fail(EVPG_ERR_ARG, "field %d cannot be uploaded", field);
    }
    const int inw = planes == 12 ? 12 : 9;
    if (count < (size_t)inw * n) return fail(EVPG_ERR_ARG, "buffer too small");
    std::vector<double> h((size_t)planes * n);
    for (size_t v = 0; v < n; v++) {
        const double* s = host + (size_t)inw * v;
        double q[12];
        if (planes == 12 || field == EVPG_F_TRANMAT) {
            memcpy(q, s, inw * sizeof(double));
        } else {
            double t[3][3];
            memcpy(t, s, sizeof t);
            if (planes == 9) tensor_to_9(t, q);
            else sym_to_b6<double>(t, q);
        }
        for (int p = 0; p < planes; p++) h[p * n + v] = q[p];
    }
    CK(cudaMemcpyAsync(dst, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (field == EVPG_F_SIG && c->precision == EVPG_FP32_BULK) {
        std::vector<float> hf(6 * n);
        for (size_t i = 0; i < hf.size(); i++) hf[i] = (float)h[i];
        CK(cudaMemcpyAsync(c->sig32, hf.data(), hf.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    return EVPG_OK;
}

}  // extern "C"
