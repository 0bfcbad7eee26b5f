// Launch arguments of every kernel of the equilibrium iteration and of the
// increment head and tail. One set per RVE context is built when the context
// is created; a single-RVE launch passes it by value (__grid_constant__), a
// batched launch reads the set of each RVE from a device table.
#pragma once
#include "evpg_common.cuh"

namespace evpg {

constexpr int NPART_NR = 15;   // err_e, err_s, sig6 sum, sig6 phase-1 sum, NR iterations
constexpr int NPART_END = 19;  // rho_F, rho_P, rho_s, rho_m, d_dipole, d_forest, d_inplane,
                               // Eps (6), Edot (5), rho_g
// Per-phase GND constants in one device row (first-order GND densities):
// |n_i . b_j| and its sine, |n_i . (n_j x b_j)| and its sine (init.c:1119-1140)
// as [NS][NS] tables, then the sense vectors b x n (init.c:198-203).
constexpr int GP_COS1 = 0, GP_SIN1 = 144, GP_COS2 = 288, GP_SIN2 = 432, GP_BP = 576,
              GP_STRIDE = 612;
constexpr int NR_BLOCK = 64;
// FP32 NR constants, one 32-byte record per (voxel, slip system): Schmid
// vector (5), passing stress, 1/(tau0 + tau_cut), gamma0_dot. Records of a
// block of NR_BLOCK voxels are contiguous ([system][voxel in block][8]), so a
// block's 24 KB arrive in shared memory by bulk copies; the two 16-byte
// halves of a record are swapped for voxels with bit 2 of their position set,
// which makes the 128-bit shared-memory reads of a warp conflict-free.
constexpr int NRC_REC = 8;
constexpr int NRC_BLOCK_FLOATS = NS * NR_BLOCK * NRC_REC;
__host__ __device__ __forceinline__ size_t nrc_index(int v, int i, int half) {
    const int b = v / NR_BLOCK, t = v - b * NR_BLOCK;
    return (((size_t)b * NS + i) * NR_BLOCK + t) * NRC_REC + 4 * (half ^ ((t >> 2) & 1));
}
constexpr int MACRO_BLOCKS = 64;
constexpr int END_BLOCK = 128;
constexpr int SPEC_THREADS = 256;
// per-orientation table row: S_gr (36), packed S066 + sym(S_gr) (21), padding
constexpr int SGR_STRIDE = 64;

// Which RVEs a launch works on, decided on the device from the RVE's Macro:
//   GATE_ALWAYS   every launch
//   GATE_RUNNING  the equilibrium loop of the increment is running and not done
//   GATE_ENDING   the loop finished without error and the tail has not run yet
//   GATE_BEGIN    a new increment was requested (IncrCtl.phase == 1)
enum Gate { GATE_ALWAYS = 0, GATE_RUNNING = 1, GATE_ENDING = 2, GATE_BEGIN = 3 };

// IncrCtl.phase
enum SlotPhase { PH_IDLE = 0, PH_BEGIN = 1, PH_RUNNING = 2, PH_ENDED = 3 };

__device__ __forceinline__ bool gate_open(const Macro* m, int gate) {
    switch (gate) {
        case GATE_RUNNING: return m->ctl.phase == PH_RUNNING && !m->done;
        case GATE_ENDING: return m->ctl.phase == PH_RUNNING && m->done && m->status == 0;
        case GATE_BEGIN: return m->ctl.phase == PH_BEGIN;
        default: return true;
    }
}

template <typename T> struct GreenK {
    T c0[3][3][3][3];
    T s0[3][3][3][3];
    int elast_bc;
    T rn[3];   // (T)(1.0 / n_a), the reference's k-vector scaling (init.c:780-797)
};

template <typename T> struct ZArgs {
    Grid g;
    FftPlan pl;
    const Macro* macro;
    int gate;
    const T* sig;        // [6][N] real
    T* dg;               // [9][N] real (inverse pass)
    C2<T>* spec;         // [9][Nh]
    const C2<T>* tw;
    const double* dE9;   // macro correction added in the inverse pass
    int P;
    T invN;
    FastDiv dn, dnh;     // divisors n2 and nh of the copy loops
};

template <typename T> struct YArgs {
    Grid g;
    FftPlan pl;
    const Macro* macro;
    int gate;
    C2<T>* spec;
    const C2<T>* tw;
    int ncomp, P;
    FastDiv dnp[2];      // np of full tiles ([0], np = P) and of the last tile ([1])
};

template <typename T> struct XArgs {
    Grid g;
    FftPlan pl;
    const Macro* macro;
    int gate;
    C2<T>* spec;
    const C2<T>* tw;
    int P;
    GreenK<T> gk;
    // index divisors: n0, and np, n0*np for full tiles ([0], np = P) and the
    // last tile ([1], np = nh - (tiles - 1) P); nh (warp-register pass)
    FastDiv dn, dnp[2], dnnp[2], dnh;
    // warp-register pass only. XM_ALL: nine components inverse-transformed
    // along x. XM_DEFER: the antisymmetric three (A12, A13, A23), needed only
    // at the end of the increment, are stored untransformed in the pass's lane
    // order (the pending buffer; the inverse plane pass adds it to the sum),
    // six inverse-transformed. XM_FLUSH: the sum inverse-transformed along x
    // into components 6..8 of spec.
    int mode;
    C2<T>* dbuf;         // [3][n1*nh pencils][n0] lane order: pending (XM_DEFER) or sum (XM_FLUSH)
};
enum XMode { XM_ALL = 0, XM_DEFER = 1, XM_FLUSH = 2 };

template <typename T> struct NrArgs {
    Material<T> mat;
    Grid g;
    T* sig;               // [6][N] lambda in, sigma out
    const T* dg;          // [9][N] strain source ([0..5] used)
    const T* epsb;        // [6][N] a = epsb - dg: Eps (FP64) or Eps - eps_begin (FP32)
    const T* schm;        // [60][N]
    const T* fc;          // [48][N]
    const float* nrc;     // FP32 sweeps: per-block NR constants (nrc_index)
    const int32_t* orient;
    const int32_t* phase;
    const T* sgr;         // [n_orient][SGR_STRIDE]
    T* edot;              // [5][N] or null
    T* gamdot;            // [12][N] or null
    Macro* macro;
    double* part;         // [warps][NPART_NR]
    T tol;
    int itmax, nr_mode;
    int stale_mode;       // 1: the first flow-rule call of the increment uses the stored rho_m
    int gate;
    // 1 (FP32-bulk form: loop sweep and FP64 refinement): a line-search Newton step
    // that already meets the NR tolerance is taken whole, without the trial
    // evaluation of its merit
    int quick_accept;
    // 1 (FP64 refinement of the FP32-bulk form): corrections with an FP32
    // Jacobian from the FP32 constant records (nrc) on FP64 residuals
    int mixed;
};

struct MacroArgs {
    LoopCfg cfg;
    Macro* macro;
    const double* part;   // [nrows][NPART_NR] warp partials of the NR sweep
    int nrows;
    double* part2;        // [MACRO_BLOCKS][NPART_NR]
    unsigned int* ticket; // last-block detection, reset by the last block
    int f32rows;          // 1: rows hold float pairs (hi, lo) of the FP32 sweep, else doubles
    int nblk;             // blocks of the first level (<= MACRO_BLOCKS, ~32 rows per block)
};

struct BeginArgs {
    Material<double> mat;
    Grid g;
    Macro* macro;        // increment controls (udot, creep, drx) in macro->ctl
    int gate;
    double* dg64;        // [9][N]
    double* dg_old;      // [9][N]
    const double* tranmat;
    const double* rho_s;
    const double* rho_m;
    const int32_t* phase;
    double* schm64;      // [60][N]
    double* fc64;        // [48][N]
    // FP32 bulk
    float* schm32;
    float* fc32;
    float* nrc32;        // FP32 NR constants (nrc_index), or null
    float* acc;          // deferred antisymmetric spectrum (zeroed here), or null
    int acc_floats;
    float* b6_32;
    float* ddg32;
    const double* epsp;
    // first-order GND densities (nullptr when off): [24][N] rho_g1, rho_g2
    const double* rho_g;
    const double* gproj;  // [2][GP_STRIDE]
    // FP32 bulk without GND (k_begin<float>): Schmid vectors and flow constants
    // computed in FP32 from these phase constants (their FP64 copies, for the
    // refinement sweep and the increment tail, are the FP32 values widened)
    PhaseK<float> ph32[2];
};

struct FoldArgs {
    Grid g;
    const Macro* macro;
    int gate;
    double* dg64;
    const float* ddg32;
    double* sig64;
    const float* sig32;
};

struct EndArgs {
    Material<double> mat;
    Grid g;
    const Macro* macro;   // tail flags in macro->ctl
    int gate;
    double udot_a[3][3];
    double* dg_old;       // in: DisGrad at increment start; out: VelGrad
    const double* dg64;
    double* epsp;
    const double* edot;
    double* tranmat;
    double* rho_s;
    double* rho_m;
    const double* gamdot;
    double* gam_acum;
    const double* sig64;
    const double* schm64;
    const int32_t* phase;
    float* sig32;         // FP32 bulk: next increment starts from the refined stress
    double* part;
    // first-order GND densities (nullptr when off)
    double* rho_g;        // [24][N] rho_g1, rho_g2
    const double* gproj;  // [2][GP_STRIDE]
    const uint8_t* gbm;   // [N] same-grain neighbour bits (x+, x-, y+, y-, z+, "z-")
    double l0;            // L0
    // FP32 bulk without GND (k_end<float>): orientation and density rates in
    // FP32 from these phase constants, the state updates in FP64
    const float* schm32;  // FP32 Schmid vectors [60][N]
    PhaseK<float> ph32[2];
};

struct EndReduceArgs {
    Macro* macro;
    int gate;
    const double* part;
    int nblocks;
    double wgt;
};

// Fused z and y passes: one CTA per (x plane, component pair), warp-register
// FFTs along z and y, the plane's half spectra staged in shared memory.
constexpr int PLANE_THREADS = 512;
constexpr int PLANE_MIN_BLOCKS = 2;  // FP32: two CTAs (one plane of one component each) per SM
constexpr int PLANE_WARPS = PLANE_THREADS / 32;

template <typename T> struct PlaneArgs {
    Grid g;
    const Macro* macro;
    int gate;
    const T* sig;        // [6][N] real (forward)
    T* dg;               // [9][N] real (inverse, += correction)
    C2<T>* spec;         // [9][Nh]
    const C2<T>* twz;    // W_n2^t
    const C2<T>* twy;    // W_n1^t
    const double* dE9;   // macro correction added in the inverse pass
    T invN;
    int nhp;             // row length of the shared-memory planes (odd, >= nh)
    FastDiv dnh;         // divisor nh of the plane copy loops
    // inverse pass: components c0 .. c0+nc-1 of every x plane (all nine, the
    // six symmetric ones when the antisymmetric part is deferred, or the three
    // deferred ones at the end of the increment). With the part deferred, the
    // pass of each iteration also adds the X pass's pending antisymmetric
    // spectrum to its sum (flat, in slices over the CTAs; ncommit complex
    // values) and CTA 0 adds dE9[6..8] to dE9_acc (the uniform part).
    int nc, c0;
    double* dE9_acc;
    C2<T>* acc;
    const C2<T>* pend;
    int ncommit;
};

// Everything one RVE context launches, with grid sizes and dynamic shared
// memory, in the context's working precision T.
template <typename T> struct SpecSet {
    ZArgs<T> z;
    YArgs<T> yf, yi;
    XArgs<T> x;
    int grid_z, grid_y, grid_x;
    size_t sm_z, sm_y, sm_x;
    // fused z+y passes (epl = n2/32 = n1/32 elements per lane; 0: not used)
    PlaneArgs<T> pl;
    int epl;
    int grid_pf, grid_pi;
    size_t sm_p;
    // warp-register X pass (xw = n0/32 elements per lane; 0: shared-memory pass)
    int xw, grid_xw;
    size_t sm_xw;
    // FP32 with the warp-register X pass and the fused plane kernels: the
    // antisymmetric part of the correction is accumulated in the spectrum and
    // transformed once, at the end of the increment (xfl, pfl)
    int defer;
    XArgs<T> xfl;
    PlaneArgs<T> pfl;
    int grid_pfl;
};

template <typename T> struct NrSet {
    NrArgs<T> a;
    int grid;
};

struct KernelSets {
    SpecSet<double> s64;
    SpecSet<float> s32;
    NrSet<double> nr64;   // loop sweep (FP64 form) or refinement (FP32 bulk)
    NrSet<float> nr32;    // loop sweep (FP32 bulk)
    MacroArgs mac;
    BeginArgs beg;
    FoldArgs fold;
    EndArgs end;
    EndReduceArgs endr;
    int grid_begin, grid_fold, grid_end;
};

}  // namespace evpg
