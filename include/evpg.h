/*
 * evpg.h -- C ABI of the GB300 EVP-FFT equilibrium iteration.
 *
 * The reference has no plugin or operator API: its hot path is a set of
 * functions sharing extern globals inside Evolution() (evolution.c:667-1551).
 * Each entry point below replaces one of those call sites, in the order the
 * reference's increment loop makes them:
 *
 *   SetupJob (init.c:728-1216)          -> evpg_job_open / evpg_create
 *   increment head (evolution.c:1030-1148, update_schmid kinematics.c:430-463)
 *                                        -> evpg_increment_begin
 *   one pass of the while loop at evolution.c:1150-1260: 9 forward FFTs
 *   (fftwnd_mpi, evolution.c:1163), Green contraction (evolution.c:1169-1183),
 *   9 inverse FFTs + DisGrad update (evolution.c:1189-1201), UpdateStress
 *   (evolution.c:157-427), error Allreduce (evolution.c:1227-1234), get_smacro
 *   (evolution.c:590-664) and the normalisation (evolution.c:1246-1252)
 *                                        -> evpg_equilibrium_iteration
 *   the whole while loop                 -> evpg_equilibrium_solve
 *   increment tail (evolution.c:1266-1362: VelGrad, Eps, averages,
 *   update_orient constitutive.c:196-273, DislocationEvolution
 *   constitutive.c:1353-1529, AvgDislocation constitutive.c:1681-1808)
 *                                        -> evpg_increment_end
 *   Evolution() itself                   -> evpg_job_run
 *   Write*MPI field dumps (io.c:283-995) -> evpg_download + evpg_job_run
 *   DestroyJob (init.c:1218-1416)        -> evpg_destroy / evpg_job_close
 *
 * Conventions: plain C types only; every call returns an evpg_status and never
 * aborts (the reference's assert/PError/exit paths become status codes);
 * device memory belongs to the context, host buffers to the caller; calls on
 * one context are ordered on its CUDA stream and a context is used by one
 * host thread at a time. Contexts are independent of each other.
 */
#ifndef EVPG_H
#define EVPG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EVPG_NSYS 12 /* NSYSMX, evpFlags.h:5 */

typedef enum evpg_status {
    EVPG_OK = 0,
    EVPG_ERR_ARG = 1,        /* bad argument, size or unsupported option */
    EVPG_ERR_CUDA = 2,       /* CUDA runtime failure (message via evpg_last_error) */
    EVPG_ERR_NOMEM = 3,      /* device or host allocation failed */
    EVPG_ERR_NAN = 4,        /* NaN in the flow rule (reference: assert, constitutive.c:624-718) */
    EVPG_ERR_SINGULAR = 5,   /* singular 6x6 system (reference: exit(35), kinematics.c:306-313) */
    EVPG_ERR_LINESEARCH = 6, /* line search found no descent (reference: PError 1203, evolution.c:324-328) */
    EVPG_ERR_ITERMAX = 7,    /* equilibrium loop hit IterMax (the reference continues silently) */
    EVPG_ERR_IO = 8,         /* input file missing or malformed */
    EVPG_ERR_NO_DEVICE = 9   /* no CUDA device */
} evpg_status;

typedef enum evpg_precision {
    EVPG_FP64 = 0,     /* plain form: every field and kernel in FP64 */
    EVPG_FP32_BULK = 1 /* NR/FFT/Green in FP32; FP64 macro BC, norms, state, final NR */
} evpg_precision;

typedef enum evpg_nr_mode {
    EVPG_NR_PLAIN = 0,      /* Newton update sigma -= J^-1 R (evolution.c:372-377) */
    EVPG_NR_LINESEARCH = 1  /* NR_MODIFIED backtracking line search (evolution.c:280-371) */
} evpg_nr_mode;

/* Per-phase material constants as SetupJob prepares them. */
typedef struct evpg_phase_desc {
    int32_t crystal;                  /* !Type_phases[p]: 1 crystal, 0 gas */
    int32_t n_sys;                    /* nSYS[p] */
    double schm_xt[EVPG_NSYS][5];     /* Schm_xt, 5-component B basis (init.c:205-212) */
    double bn[EVPG_NSYS][3];          /* unit slip normals, crystal frame */
    double bb[EVPG_NSYS][3];          /* unit slip directions, crystal frame */
    double burgers[EVPG_NSYS];        /* bb_B [nm] */
    double chi[EVPG_NSYS][EVPG_NSYS];  /* Chi (self + coplanar) */
    double chi1[EVPG_NSYS][EVPG_NSYS]; /* Chi_1 (cross, glissile, Hirth, Lomer) */
    double shear_g;                   /* Shear_G [MPa] */
    double c1, c2, c3, c4, c5, c6;    /* C_1..C_6 */
    double q_slip, q_bulk;            /* Q * MY_J_IN_EV / kT (constitutive.c:543, 1381) */
    double tau0;                      /* lattice resistance tau0xf (constitutive.c:537) */
} evpg_phase_desc;

/* The RVE and its set-up state. Host arrays are read during evpg_create only. */
typedef struct evpg_rve_desc {
    int32_t n[3];                 /* CellDim */
    int32_t n_orient;             /* rows of c_gr / s_gr */
    const int32_t *voxel_orient;  /* [N] row of c_gr/s_gr, -1 for gas voxels */
    const int32_t *voxel_phase;   /* [N] phase id, 1 or 2 (phase_f) */
    const double *c_gr;           /* [n_orient][6][6] C_gr (B basis, sample frame) */
    const double *s_gr;           /* [n_orient][6][6] LU inverse of c_gr */
    const double *tranmat;        /* [N][3][3] TranMat_xt2sa */
    const double *sig0;           /* [N][3][3] initial stress (InitFields, init.c:470-492) */
    const double *rho_s0;         /* [N][12] initial SSD density [1e12 m^-2] */
    double c066[6][6], s066[6][6];  /* C066 = <C_gr>, S066 = LU inverse */
    double c0[3][3][3][3];        /* C0 (reference stiffness for the Green operator) */
    double s0[3][3][3][3];        /* S0 (k=0 term with ElastBC 0; mixed-BC update) */
    double wgt_ph1;               /* Wgt_ph1 */
    evpg_phase_desc phase[2];
    double dt;                    /* TimeStep [s] */
    double kT;                    /* T__K*BOLZ*J_IN_EV [eV] */
    double temperature;           /* T__K */
    double nu;                    /* ElastConst_PhaseI[3] */
    double d0;                    /* D_0 */
    double delta_tau_drx;         /* DeltaTau_DRX */
    double tau_drx;               /* tau_DRX */
    int32_t elast_bc;             /* ElastBC */
    int32_t velgrad_bc_flag[6];   /* VelGrad_BC_Flag (Voigt 11,22,33,23,13,12) */
    int32_t stress_bc_flag[6];    /* Stress_BC_Flag */
    double scauchy[3][3];         /* applied Cauchy stress */
    double udot_a[3][3];          /* antisymmetric part of the applied velocity gradient */
    double err_tol;               /* Err */
    int32_t iter_max;             /* IterMax */
    int32_t precision;            /* evpg_precision */
    int32_t nr_mode;              /* evpg_nr_mode */
} evpg_rve_desc;

/* Macro quantities after an equilibrium iteration (all FP64). */
typedef struct evpg_iter_out {
    double err_e, err_s;          /* normalised errors (evolution.c:1246-1252) */
    double err_e_sum, err_s_sum;  /* sum over voxels before normalisation */
    double sig_avg[3][3];         /* SigAvg */
    double sig_avg_ph1[3][3];     /* SigAvg1 */
    double ddisgrad[3][3];        /* dDisGradAvg of this iteration */
    double ddisgrad_acum[3][3];   /* dDisGradAvg_acum */
    double s_vm, s_vm1;
    int32_t iter;                 /* iterations run in the current increment */
    int32_t converged;
} evpg_iter_out;

/* Increment tail outputs (evolution.c:1307-1332, constitutive.c:1681-1808). */
typedef struct evpg_incr_out {
    double eps_avg[3][3], edot_avg[3][3];
    /* rho_F, rho_P, rho_s, rho_m, rho_g, rho_dipole, rho_forest, rho_inplane */
    double rho_avg[8];
    int64_t nr_iterations;        /* NR iterations summed over voxels and sweeps */
} evpg_incr_out;

/* Fields for evpg_download / evpg_upload, [N][...] voxel-major, double. */
typedef enum evpg_field {
    EVPG_F_SIG = 0,        /* [N][3][3] Sig */
    EVPG_F_DISGRAD = 1,    /* [N][3][3] DisGrad */
    EVPG_F_EPS = 2,        /* [N][3][3] Eps (plastic strain) */
    EVPG_F_EDOT = 3,       /* [N][3][3] Edot */
    EVPG_F_TRANMAT = 4,    /* [N][3][3] TranMat_xt2sa */
    EVPG_F_RHO_S = 5,      /* [N][12] rho_s */
    EVPG_F_RHO_M = 6,      /* [N][12] rho_m */
    EVPG_F_GAMDOT = 7,     /* [N][12] gamdot */
    EVPG_F_GAM_ACUM = 8,   /* [N][12] gam_acum */
    EVPG_F_VELGRAD = 9,    /* [N][3][3] VelGrad (valid after evpg_increment_end) */
    EVPG_F_SIG6 = 10       /* [N][6] Sig in .iout order 11,22,33,23,13,12 */
} evpg_field;

const char *evpg_version(void);
const char *evpg_status_string(int status);
/* Message of the last error on this host thread. */
const char *evpg_last_error(void);

int evpg_create(const evpg_rve_desc *desc, void **ctx_out);
int evpg_destroy(void *ctx);
/* Use an existing cudaStream_t for all work of this context (NULL: own stream). */
int evpg_set_stream(void *ctx, void *cuda_stream);
int evpg_device_bytes(void *ctx, int64_t *bytes);

/* Increment head: VelGrad <- DisGrad, DisGrad += udot_dt (the applied
 * velocity gradient times TimeStep, evolution.c:1115-1128; with creep = 1 the
 * field is set to disgrad_avg_actual instead), update_schmid, reset of the
 * macro corrections and errors. time_tot is TimeTot during the increment. */
int evpg_increment_begin(void *ctx, const double udot_dt[3][3], int32_t creep,
                         const double disgrad_avg_actual[3][3], double time_tot);

/* One equilibrium iteration with the device-side get_smacro. e_vm is the
 * normaliser of the strain error for this increment. out may be NULL. */
int evpg_equilibrium_iteration(void *ctx, double e_vm, evpg_iter_out *out);

/* The whole equilibrium loop on the device until max(|Err_s|,|Err_e|) <= Err
 * or IterMax; out may be NULL. Returns EVPG_OK also when IterMax is reached
 * (out->converged tells), as the reference does. */
int evpg_equilibrium_solve(void *ctx, double e_vm, evpg_iter_out *out);

/* Increment tail. update_orient runs when reorient != 0 (the reference:
 * Update_Flag == 1 && istep > 1). out may be NULL. */
int evpg_increment_end(void *ctx, int32_t reorient, evpg_incr_out *out);

int evpg_download(void *ctx, int32_t field, double *host, size_t count);
int evpg_upload(void *ctx, int32_t field, const double *host, size_t count);
int evpg_synchronize(void *ctx);

/* Optional per-kernel timing with CUDA events on the context's stream
 * (no counterpart in the reference). Groups, in order: forward z, forward y,
 * x pass with the Green contraction, inverse y, inverse z with the DisGrad
 * update, NR sweep, macro update, increment head, increment tail, FP64
 * refinement sweep. evpg_profile resets the totals; while profiling, the
 * equilibrium loop checks convergence after every iteration. */
#define EVPG_PROFILE_GROUPS 10
int evpg_profile(void *ctx, int32_t enable);
int evpg_profile_read(void *ctx, double *ms, int64_t *launches, int32_t n);
/* Kernels launched on this context so far. */
int evpg_launch_count(void *ctx, int64_t *n);

/* Allocation-free Green-operator correction (no counterpart in the
 * reference). For callers that cannot allocate device memory on the call
 * path -- their device memory belongs to another allocator, or their device
 * footprint is fixed when the library loads. It computes, in FP64,
 *   du9 = Re IFFT( Gamma(k) : FFT(sig6) ) / N
 * the displacement-gradient correction of one equilibrium iteration
 * (evolution.c:1157-1201 without the macro term), from caller-owned device
 * buffers: sig6 [6][N] is the stress in the B basis (one plane per
 * component, voxel index (x*n1+y)*n2+z), du9 [9][N] receives the B basis of
 * the symmetric part and A12, A13, A23 of the antisymmetric part. c0 and s0
 * are C0 and S0 (3x3x3x3, row-major); elast_bc is ElastBC.
 * Limits: every n_i <= 64 and n0*n1*(n2/2+1) <= 17408 (e.g. 32^3); larger
 * grids return EVPG_ERR_ARG. Scratch is a static device array of ~2.5 MB that
 * every GPU loading the library keeps until exit; nothing is allocated. The
 * first call on a device looks up that array's device address, so make that
 * first call outside any stream capture. Calls whose work overlaps on the GPU
 * share the array and race: serialise them. stream: a cudaStream_t or NULL. */
int evpg_green_correction_noalloc(const double *sig6, double *du9, int32_t n0, int32_t n1,
                                  int32_t n2, const double c0[81], const double s0[81],
                                  int32_t elast_bc, void *stream);

/* ---- host driver: the reference's own input files and increment loop ---- */

/* GetNameList + SetupJob from the reference's namelist file; relative file
 * names inside it are resolved against the namelist's directory. rho0_path
 * (nullable) holds N doubles of initial SSD density, one per voxel, applied
 * to every slip system. precision: evpg_precision; nr_mode: evpg_nr_mode. */
int evpg_job_open(const char *input_path, const char *rho0_path, int32_t precision,
                  int32_t nr_mode, void **job_out);
int evpg_job_close(void *job);
void *evpg_job_ctx(void *job);
int evpg_job_nvox(void *job, int32_t n[3]);
int evpg_job_nsteps(void *job);

/* One increment of Evolution() (evolution.c:726-1520) on the device.
 * iters: equilibrium iterations taken. */
int evpg_job_increment(void *job, int32_t istep, int32_t *iters);

/* Scalars after the last increment: [0] TimeTot, [1] e_vm, [2] evmp,
 * [3] d_vm, [4] dvmp, [5] s_vm, [6] s_vm1, [7..15] SigAvg, [16..24] SigAvg1,
 * [25..32] rho averages as evpg_incr_out, [33] NR iterations of the
 * increment. */
int evpg_job_scalars(void *job, double *out, int32_t count);

/* Evolution() into outdir: vm.out, dd.out, err.out, iters.txt, and with
 * write_iout the reference's .iout dumps at PrintControl steps. nsteps < 0:
 * N_steps from the namelist. */
int evpg_job_run(void *job, const char *outdir, int32_t nsteps, int32_t write_iout);

#ifdef __cplusplus
}
#endif
#endif
