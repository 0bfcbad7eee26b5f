// Device context of one RVE and the launchers of its kernels.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include "evpg_common.cuh"

namespace evpg {

constexpr int NPART_NR = 15;   // err_e, err_s, sig6 sum, sig6 phase-1 sum, NR iterations
constexpr int NPART_END = 18;  // rho_F, rho_P, rho_s, rho_m, d_dipole, d_forest, d_inplane,
                               // Eps (6), Edot (5)
constexpr int NR_BLOCK = 128;
constexpr int MACRO_BLOCKS = 64;
constexpr int END_BLOCK = 128;

// Kernel groups timed by the optional profiler (CUDA events on the context's
// stream around each launch).
enum ProfGroup { PG_FWD_Z, PG_FWD_Y, PG_X_GREEN, PG_INV_Y, PG_INV_Z, PG_NR, PG_MACRO,
                 PG_BEGIN, PG_END, PG_REFINE, PG_COUNT };

struct Profiler {
    bool on = false;
    struct Rec { int group; cudaEvent_t a, b; };
    Rec* recs = nullptr;
    int n = 0, cap = 0;
    double ms[PG_COUNT] = {0};
    long long launches[PG_COUNT] = {0};
};

struct Ctx {
    Grid g;
    int precision;  // 0 FP64, 1 FP32 bulk
    int nr_mode;    // 0 plain, 1 line search
    int n_orient;
    cudaStream_t stream;
    bool own_stream;
    FftPlan pl[3];  // x, y, z
    double2* tw64[3];
    float2* tw32[3];
    // FP64 state (both precisions)
    double *sig64, *dg64, *dg_old, *epsp, *edot64, *rho_s, *rho_m, *gamdot64, *gam_acum,
        *tranmat, *schm64, *fc64, *sgr64;
    int32_t *orient, *phase;
    // FP32 working set (FP32 bulk only)
    float *sig32, *ddg32, *b6_32, *schm32, *fc32, *sgr32;
    void* spec;  // 9 * Nh complex of the working precision
    double* part_nr;   // [nb_nr * NR_BLOCK/32][NPART_NR] warp partials
    int nb_nr;
    double* part_nr2;  // [MACRO_BLOCKS][NPART_NR]
    unsigned int* ticket;
    double* part_end;
    int nb_end;
    Macro* macro;       // device
    Macro* macro_host;  // pinned mirror
    LoopCfg cfg;
    Material<double> m64;
    Material<float> m32;
    double delta_tau_drx, tau_drx;
    double udot_a[3][3];
    size_t bytes;
    int nr_itmax;
    double nr_tol64, nr_tol32;
    Profiler prof;
    long long launches;  // kernels launched on this context (all groups)
};

// Record the start (begin=true) or end of a launch of `group` when profiling.
void prof_mark(Ctx& c, int group, bool begin);

// Device address of a member of the device-resident Macro struct.
template <typename F> inline F* macro_field(Macro* m, size_t off) {
    return reinterpret_cast<F*>(reinterpret_cast<char*>(m) + off);
}

template <typename T> inline const Material<T>& material_of(const Ctx& c);
template <> inline const Material<double>& material_of<double>(const Ctx& c) { return c.m64; }
template <> inline const Material<float>& material_of<float>(const Ctx& c) { return c.m32; }

// spectral chain of one iteration in the working precision
cudaError_t launch_spectral(Ctx& c);
// NR sweep: refine = 0 inside the loop (working precision), 1 the FP64
// refinement of the FP32-bulk form at the end of the loop
cudaError_t launch_nr(Ctx& c, int refine);
cudaError_t launch_macro(Ctx& c);
cudaError_t launch_begin(Ctx& c, const double udot9[9], int creep, const double dgavg9[9],
                         double drx);
cudaError_t launch_fold(Ctx& c);
cudaError_t launch_end(Ctx& c, int reorient);

}  // namespace evpg
