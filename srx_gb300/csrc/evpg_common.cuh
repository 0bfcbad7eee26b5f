// Shared device definitions of the EVP-FFT kernels.
//
// Field layout in HBM (structure of arrays, one plane of N values per
// component, voxel index v = (x*n1 + y)*n2 + z as the reference's pIDX,
// evp.h:60):
//   sig    [6][N]  Cauchy stress in the Lebensohn-Tome B basis
//                  (kinematics.c:14-54; component 6 is hydrostatic)
//   dg     [9][N]  displacement gradient: [0..5] B basis of its symmetric
//                  part (the NR's strain), [6..8] antisymmetric part A12,A13,A23
//   spec   [9][n0*n1*(n2/2+1)] complex half spectrum (z halved)
// State that only changes once per increment is FP64 in both precisions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace evpg {

constexpr int NS = 12;  // slip systems per phase (NSYSMX)

// kinematics.c:22-24 (the B-basis constants as the reference writes them)
constexpr double RSQ2 = 0.70710678118654744;
constexpr double RSQ3 = 0.57735026918962584;
constexpr double RSQ6 = 0.40824829046386304;

template <typename T> struct cplx_t;
template <> struct cplx_t<double> { using type = double2; };
template <> struct cplx_t<float> { using type = float2; };
template <typename T> using C2 = typename cplx_t<T>::type;

template <typename T> __host__ __device__ __forceinline__ C2<T> mk(T x, T y) {
    C2<T> r; r.x = x; r.y = y; return r;
}
template <typename T> __device__ __forceinline__ C2<T> cadd(C2<T> a, C2<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ C2<T> csub(C2<T> a, C2<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ C2<T> cmul(C2<T> a, C2<T> b) {
    return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> __device__ __forceinline__ C2<T> cscale(C2<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
template <typename T> __device__ __forceinline__ C2<T> cconj(C2<T> a) { return mk<T>(a.x, -a.y); }

// B-basis 6-vector -> symmetric tensor (chg_basis opt 1) and back (opt 2),
// written out for the sparse B matrices.
template <typename T> __host__ __device__ __forceinline__ void b6_to_sym(const T* v, T s[3][3]) {
    const T r2 = (T)RSQ2, r3 = (T)RSQ3, r6 = (T)RSQ6;
    s[0][0] = -r2 * v[0] - r6 * v[1] + r3 * v[5];
    s[1][1] = r2 * v[0] - r6 * v[1] + r3 * v[5];
    s[2][2] = (T)2 * r6 * v[1] + r3 * v[5];
    s[1][2] = s[2][1] = r2 * v[2];
    s[0][2] = s[2][0] = r2 * v[3];
    s[0][1] = s[1][0] = r2 * v[4];
}
template <typename T> __host__ __device__ __forceinline__ void sym_to_b6(const T s[3][3], T* v) {
    const T r2 = (T)RSQ2, r3 = (T)RSQ3, r6 = (T)RSQ6;
    v[0] = -r2 * s[0][0] + r2 * s[1][1];
    v[1] = -r6 * s[0][0] - r6 * s[1][1] + (T)2 * r6 * s[2][2];
    v[2] = r2 * (s[1][2] + s[2][1]);
    v[3] = r2 * (s[0][2] + s[2][0]);
    v[4] = r2 * (s[0][1] + s[1][0]);
    v[5] = r3 * (s[0][0] + s[1][1] + s[2][2]);
}

// Per-phase constants with the flow rule's products folded
// (constitutive.c:585-692). All derived on the host in FP64.
template <typename T> struct PhaseK {
    int crystal, n_sys;
    T chi[NS][NS], chi1[NS][NS];
    T k_tpass[NS];   // c1*G*b*1e-3        -> tau_pass = k*sqrt(|rho_P+rho_m|)
    T k_tcut[NS];    // (kT/0.624)/c2/c3/b/b*0.1 -> tau_cut = k*sqrt(rho_f)
    T k_rhom[NS];    // 2kT/c1/c2/c3/G/b^3*160.2177 -> rho_m = k*sqrt(rho_P*rho_f)
    T k_gamo[NS];    // 1e-3*1e10*c2*b*exp(-q_slip) -> gam_o = k*rho_m/sqrt(rho_f)
    // DislocationEvolution prefixes (constitutive.c:1401-1403): d_dipole =
    // k_ddip/(|rss|+1e-4) (left to right as there)
    T k_ddip[NS];    // sqrt(3)*G*b/16/pi/(1-nu)
    T k_hyd[NS];     // G*b/pi/(1-nu)
    T k_d0b[NS];     // D_0/b
    // one division per system instead of three: hydro = k_hydr (|rss| + 1e-4)
    // with k_hydr = k_hyd / k_ddip, and the exponent |hydro| k_hexp with
    // k_hexp = b^3 100 / (1.38 T)
    T k_hydr[NS];
    T k_hexp[NS];
    T tau0;
    T schm_xt[NS][5];
    T bn[NS][3], bb[NS][3];
    T burgers[NS];
    T shear_g, c4, c5, c6, q_bulk;
};

// Everything the per-voxel kernels need about the material and load, passed
// by value (__grid_constant__) so reads hit the constant bank.
template <typename T> struct Material {
    PhaseK<T> ph[2];
    T c066[6][6], s066[6][6];  // C066, S066 (B basis)
    T c0[3][3][3][3], s0[3][3][3][3];
    T dt, kT, temperature, nu, d0;
    int elast_bc;
};

// Controls of the next increment, written by the host (one stream-ordered
// copy) before the increment head runs.
struct IncrCtl {
    double udot9[9];    // applied Udot*dt in the field representation
    double dgavg9[9];   // uniform DisGrad for creep
    double drx;         // DeltaTau_DRX*exp(...) of this increment
    double e_vm;        // strain-error normaliser of this increment
    double err0;        // initial error value (2*Err)
    int creep;
    int tail;           // increment-tail flags: 1 update_orient, 2 GND slip-rate gradients
    int phase;          // 0 idle, 1 begin requested, 2 running, 3 ended
    int pad;
};

// Device-resident macro state of the equilibrium loop (always FP64).
struct Macro {
    IncrCtl ctl;
    double dE[3][3];        // dDisGradAvg of the last iteration (upper triangle)
    double dE9[9];          // the same in the field representation (B basis + A12,A13,A23)
    double dE9_acc[9];      // deferred antisymmetric part: sum of the dE9[6..8] applied so far
    double dE_acum[3][3];   // dDisGradAvg_acum
    double sig_avg[3][3], sig_avg1[3][3];
    double err_e, err_s, err_e_sum, err_s_sum;
    double s_vm, s_vm1;
    double e_vm;            // strain-error normaliser of this increment
    double tpass_drx;       // DeltaTau_DRX*exp(...) for this increment
    int iter;               // equilibrium iterations in this increment
    int done;               // converged or IterMax reached
    int converged;
    int status;             // sticky kernel error (EVPG_ERR_*)
    long long nr_iters;     // NR iterations summed over voxels (this increment)
    // increment tail
    double eps_avg6[6], edot_avg6[6];
    double rho_avg[8];
    double rho_dip_acc, rho_for_acc, rho_inp_acc;  // running sums of the increments
};

// Static configuration of the BC and loop control (FP64).
struct LoopCfg {
    double s0[3][3][3][3];
    double scauchy[3][3];
    int vflag[6], sflag[6];
    double wgt, wgt_ph1;
    double err_tol;
    int iter_max;
};

// Sizes and pointers of one context used by several kernels.
struct Grid {
    int n0, n1, n2, nh;   // nh = n2/2 + 1
    int N;                // n0*n1*n2
    long long Nh;         // n0*n1*nh
};

// Stockham FFT plan for one axis length.
// Division by a divisor d >= 1 fixed per launch, for dividends below 2^24,
// as a multiply and shift: q = (x * m) >> s with s = 24 + ceil(log2 d) and
// m = ceil(2^s / d) < 2^25 + 1. Exact: x m / 2^s exceeds x / d by less than
// 2^24 d / (d 2^s) <= 1/d, so the floor is unchanged. Replaces the
// integer-divide sequence in the index arithmetic of the FFT loops.
struct FastDiv {
    unsigned long long m;
    int s;
    __host__ __device__ void set(int d) {
        int l = 0;
        while ((1 << l) < d) l++;
        s = 24 + l;
        m = ((1ull << s) + (unsigned long long)d - 1) / (unsigned long long)d;
    }
    __device__ __forceinline__ int div(int x) const {
        return (int)(((unsigned long long)(unsigned)x * m) >> s);
    }
};

struct FftPlan {
    int n, nf;
    int radix[12];
    int ns[12];
    FastDiv dm[12], dns[12];  // n / radix[s] and ns[s]
};

// Divisors of every stage, after radix[] and ns[] are set.
inline void plan_divisors(FftPlan& p) {
    for (int s = 0; s < p.nf; s++) {
        p.dm[s].set(p.n / p.radix[s]);
        p.dns[s].set(p.ns[s]);
    }
}

}  // namespace evpg
