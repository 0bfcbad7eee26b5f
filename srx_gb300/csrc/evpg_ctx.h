// Device context of one RVE and the launchers of its kernels.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include "evpg_args.h"

namespace evpg {

// Kernel groups timed by the optional profiler (CUDA events on the context's
// stream around each launch).
// doubles per download chunk (packed records, at most 12 per voxel); two
// chunks per buffer
constexpr size_t DL_CHUNK_DOUBLES = (size_t)1 << 22;
inline size_t dl_chunk_doubles(size_t nvox) {
    return 12 * nvox < DL_CHUNK_DOUBLES ? 12 * nvox : DL_CHUNK_DOUBLES;
}

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
    // first-order GND densities (gnd = 1 only)
    double *rho_g, *gproj;
    uint8_t* gbm;
    double l0;
    // FP32 working set (FP32 bulk only)
    float *sig32, *ddg32, *b6_32, *schm32, *fc32, *sgr32;
    float* nrc32;  // FP32 NR constants per block of NR_BLOCK voxels (nrc_index)
    void* spec;  // 9 * Nh complex of the working precision
    double* part_nr;   // [nb_nr * NR_BLOCK/32][NPART_NR] warp partials
    int nb_nr;
    double* part_nr2;  // [MACRO_BLOCKS][NPART_NR]
    unsigned int* ticket;
    double* part_end;
    int nb_end;
    Macro* macro;       // device
    Macro* macro_host;  // pinned mirror
    IncrCtl* ctl_host;  // pinned staging of the next increment's controls
    KernelSets* ks;     // launch arguments of every kernel (built at creation)
    int sched_p[3];     // pencils per CTA of the z, y, x passes (0: default)
    int sched_fused;    // fused z+y passes: -1 default (FP32 bulk when eligible), 0 off, 1 on
    int sched_xpass;    // warp-register X pass: -1 default (when eligible), 0 off, 1 on
    int nsm;            // SM count of the device
    long long version;  // bumped whenever ks changes (batches refresh their tables)
    double* dl_dev;     // download packing buffers (2 chunks, allocated on first use)
    double* dl_host;    // pinned staging (2 chunks)
    cudaEvent_t dl_ev[2];
    void* solo;         // batch of this context alone (evpg_increment's round graph)
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

// Fill c.ks from the allocated context (pencils per CTA, grids, shared memory).
void build_sets(Ctx& c);
void build_spectral_sets(Ctx& c);
void build_solver_sets(Ctx& c);
// Largest and default pencils per CTA of the z, y, x passes.
void spec_pmax(const Grid& g, size_t elem_bytes, int pmax[3]);
void spec_default_p(const Grid& g, size_t elem_bytes, int nsm, int P[3]);
// Message of the last error on this host thread (evpg_last_error); returns st.
int record_error(int st, const char* msg);
// Autotune the spectral schedule (returns 0, 2 CUDA failure, 3 no memory);
// force: search even when the grid is cached; gain: default time / tuned time.
int tune_spectral(Ctx& c, int force, double* gain);
// Release the context's own round graph.
void free_solo(Ctx& c);
// Set the kernels' dynamic shared-memory limits (once per device).
void set_kernel_attributes();
void spectral_attributes();
void solver_attributes();

// One batched launch: the per-RVE argument table (device), the CTA map
// (device, map[b] = (slot, CTA index within the slot)), the CTA count and the
// dynamic shared memory (maximum over the slots).
struct BatchLaunch {
    const void* tab;
    const int2* map;
    int nblk;
    size_t smem;
};
enum BatchKind { BL_Z, BL_YF, BL_X, BL_YI, BL_NR, BL_MACRO, BL_MBEGIN, BL_BEGIN, BL_FOLD,
                 BL_REFINE, BL_END, BL_ENDR, BL_PF1, BL_PF2, BL_PF4, BL_PI1, BL_PI2, BL_PI4,
                 BL_XW1, BL_XW2, BL_XW4, BL_BEGIN32, BL_END32, BL_XFL1, BL_XFL2, BL_XFL4,
                 BL_PFL1, BL_PFL2, BL_PFL4, BL_COUNT };
// Spectral chain of a batch: the separate z and y passes over the slots in
// BL_Z/BL_YF/BL_YI, the fused plane kernels over the slots in BL_PF*/BL_PI*
// (1, 2, 4 elements per lane), the X pass as the warp-register kernel over the
// slots in BL_XW* (1, 2, 4 elements per lane) and the shared-memory kernel over
// those in BL_X; launches with no slot are skipped. Returns the number of
// kernels launched.
// parts of the spectral chain: all passes, the forward transforms with the X
// pass (they write only the spectrum buffer), the inverse transforms
enum SpecPart { SPEC_ALL = 0, SPEC_FWD = 1, SPEC_INV = 2 };
int launch_spectral_batch(int precision, const BatchLaunch* L, cudaStream_t st, int part = SPEC_ALL);
// end-of-increment flush of the slots that defer the antisymmetric part
int launch_flush_batch(const BatchLaunch* L, cudaStream_t st);
int plane_epl(const Grid& g, size_t elem_bytes);
// NR sweep, macro update for every slot
cudaError_t launch_nr_batch(int precision, int nr_mode, const BatchLaunch& L, cudaStream_t st);
cudaError_t launch_macro_batch(const BatchLaunch& L, cudaStream_t st);
// increment head (macro reset + k_begin), gated per slot
// increment head over the slots of BL_BEGIN (FP64 arithmetic) and BL_BEGIN32
// (FP32-bulk without GND); returns the number of kernels launched
int launch_begin_batch(const BatchLaunch* L, cudaStream_t st);
// increment tail (fold + FP64 refinement for FP32 bulk, k_end, k_end_reduce)
// increment tail (FP32 fold and FP64 refinement first in the FP32-bulk form);
// returns the number of kernels launched
int launch_end_batch(int precision, int nr_mode, const BatchLaunch* L, cudaStream_t st);
// the head and tail of this context compute in FP32 (FP32 bulk without GND)
bool head_tail_fp32(const Ctx& c);

// Launchers of one RVE's kernels on its stream; `gate` selects when a launch
// does work (Gate).
// spectral chain of one iteration in the working precision
cudaError_t launch_spectral(Ctx& c, int gate, int part = SPEC_ALL);
// end of the increment (before the fold): the deferred antisymmetric part of
// the correction into DisGrad; no launch when the context does not defer it
cudaError_t launch_spectral_flush(Ctx& c, int gate);
int spectral_flush_kernels(const Ctx& c);
// NR sweep: refine = 0 inside the loop (working precision), 1 the FP64
// refinement of the FP32-bulk form at the end of the loop
cudaError_t launch_nr(Ctx& c, int refine, int gate);
cudaError_t launch_macro(Ctx& c);
// reset of the macro state at the increment head (controls from macro->ctl)
cudaError_t launch_macro_begin(Ctx& c, int gate);
cudaError_t launch_begin(Ctx& c, int gate);
cudaError_t launch_fold(Ctx& c, int gate);
cudaError_t launch_end(Ctx& c, int gate);
// macro->ctl.phase: from -> to (single thread)
cudaError_t launch_phase(Ctx& c, int from, int to);

}  // namespace evpg
