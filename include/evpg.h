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
 *   update_orient constitutive.c:196-273, the DD_GND slip-rate gradients
 *   Gradient_ShearRate constitutive.c:881-1112, DislocationEvolution
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
    EVPG_ERR_NO_DEVICE = 9,  /* no CUDA device */
    EVPG_ERR_TIMEOUT = 10    /* a device-side wait for a copy exceeded its bound (the RVE stops) */
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
    /* First-order GND densities: the reference built with DD_GND (which
     * implies DD_GND_FIRST_ORDER, evpFlags.h:29-32). Screw and edge densities
     * per slip system grow from the slip-rate gradients across each grain
     * (Gradient_ShearRate, constitutive.c:881-1112; DislocationEvolution,
     * constitutive.c:1428-1522) and enter the forest and parallel densities
     * of the flow rule (constitutive.c:558-577) and rho_tot
     * (evolution.c:1041-1045). 0 leaves them out (the shipped build). */
    int32_t gnd;                  /* 1: on */
    double l0;                    /* L0 of the namelist (> 0 when gnd = 1) */
    const int32_t *voxel_grain;   /* [N] grain ids (grain_f); read when gnd = 1 */
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
    EVPG_F_DISGRAD = 1,    /* [N][3][3] DisGrad (FP32-bulk contexts: the equilibrium loop's
                              corrections, held in FP32 during the loop, their
                              antisymmetric part summed in the spectrum, enter
                              it at evpg_increment_end; between iterations the
                              field holds the increment head's value) */
    EVPG_F_EPS = 2,        /* [N][3][3] Eps (plastic strain) */
    EVPG_F_EDOT = 3,       /* [N][3][3] Edot */
    EVPG_F_TRANMAT = 4,    /* [N][3][3] TranMat_xt2sa */
    EVPG_F_RHO_S = 5,      /* [N][12] rho_s */
    EVPG_F_RHO_M = 6,      /* [N][12] rho_m */
    EVPG_F_GAMDOT = 7,     /* [N][12] gamdot */
    EVPG_F_GAM_ACUM = 8,   /* [N][12] gam_acum */
    EVPG_F_VELGRAD = 9,    /* [N][3][3] VelGrad (valid after evpg_increment_end) */
    EVPG_F_SIG6 = 10,      /* [N][6] Sig in .iout order 11,22,33,23,13,12 */
    EVPG_F_RHO_G1 = 11,    /* [N][12] rho_g1, screw GND density (contexts with gnd = 1) */
    EVPG_F_RHO_G2 = 12     /* [N][12] rho_g2, edge GND density (contexts with gnd = 1) */
} evpg_field;

/* Flags of the increment tail (evpg_increment_end, evpg_increment,
 * evpg_batch_stage). */
typedef enum evpg_tail_flag {
    EVPG_TAIL_REORIENT = 1,    /* update_orient (Update_Flag == 1 && istep > 1) */
    EVPG_TAIL_GND_GRADIENT = 2 /* slip-rate gradients for the GND densities this increment
                                  (Hard_Flag == 1 && istep > 1, evolution.c:1348-1357);
                                  otherwise the gradients stay at their initial zeros */
} evpg_tail_flag;

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

/* Increment tail. tail: evpg_tail_flag bits (update_orient with
 * EVPG_TAIL_REORIENT, the reference's Update_Flag == 1 && istep > 1). out
 * may be NULL. */
int evpg_increment_end(void *ctx, int32_t tail, evpg_incr_out *out);

/* The whole increment -- head, equilibrium loop, tail -- as one CUDA graph
 * launch on the context's stream (captured on the first call, replayed
 * after): the loop is a conditional WHILE node whose condition the device
 * sets after every iteration, so no host round trip happens inside the
 * increment. Same results as evpg_increment_begin + evpg_equilibrium_solve +
 * evpg_increment_end (with the increment tail skipped when the loop stops on
 * an error). e_vm: strain-error normaliser; tail as in
 * evpg_increment_end. it/inc may be NULL. No counterpart in the reference,
 * whose loop is host-driven (evolution.c:1150). */
int evpg_increment(void *ctx, const double udot_dt[3][3], int32_t creep,
                   const double disgrad_avg_actual[3][3], double time_tot, double e_vm,
                   int32_t tail, evpg_iter_out *it, evpg_incr_out *inc);

/* Change the loading between increments (a mid-run BC switch, e.g.
 * tension then shear; the reference reads one BC set per run, init.c:865-901):
 * the Voigt flags, the applied Cauchy stress and the antisymmetric part of
 * the applied velocity gradient. The host passes the new Udot*dt to the next
 * increment head. No counterpart in the reference. */
int evpg_set_load(void *ctx, const int32_t velgrad_bc_flag[6], const int32_t stress_bc_flag[6],
                  const double scauchy[3][3], const double udot_a[3][3]);
/* Autotuner of the spectral schedule (no counterpart in the reference):
 * for this context's grid and precision, times the FFT radix orders of each
 * axis and the pencils per CTA of each pass on the context's own buffers
 * (state untouched) and keeps the fastest; results are cached per grid and
 * precision for the process, so later contexts of the same grid reuse them
 * (force = 1 searches again). gain (nullable) = default / tuned time of the
 * spectral passes (0 when taken from the cache). Pencil counts leave the
 * arithmetic unchanged; a different radix order changes FFT rounding only.
 * evpg_get_schedule reports pencils per CTA of the z, y, x passes and the
 * radix stages of the x, y, z axes. */
int evpg_tune(void *ctx, int32_t force, double *gain);
int evpg_get_schedule(void *ctx, int32_t pencils[3], int32_t radix[3][12], int32_t nstages[3]);
/* Relative stress-change tolerance and iteration cap of the per-voxel NR
 * (the reference: 1e-10 and 500, evolution.c:217-218). The FP64 form
 * defaults to those; the FP32-bulk loop defaults to 1e-5
 * and its final FP64 refinement keeps 1e-10. The tolerance applies to the
 * working-precision loop sweep, the cap to every sweep. */
int evpg_set_nr_tolerance(void *ctx, double tol, int32_t itmax);
/* Fused z+y passes (one x plane per CTA, warp-register FFTs along z and y;
 * n1 == n2 in {32, 64, 128} when the planes fit in shared memory): mode -1
 * default (on for FP32 bulk where eligible), 0 off, 1 on where eligible.
 * evpg_get_schedule then reports 0 pencils for the z and y passes. */
int evpg_set_fused(void *ctx, int32_t mode);
/* X pass as warp-register transforms (one warp per (y, kz) pencil with the six
 * stress components in registers, FP32 with n0 in {32, 64, 128}): mode -1
 * default (on where eligible), 0 the shared-memory Stockham pass (whose radix
 * order evpg_set_radix sets), 1 on where eligible. The autotuner times both. */
int evpg_set_xpass(void *ctx, int32_t mode);
/* FFT radix order of one axis (0 x, 1 y, 2 z) for the Stockham passes:
 * nstages radices (2..16, product n of the axis; 16 in FP32 contexts on the
 * x axis only) applied in the given order. The autotuner chooses among such
 * orders. */
int evpg_set_radix(void *ctx, int32_t axis, const int32_t *radix, int32_t nstages);
/* Spectral kernels the context runs (no counterpart in the reference):
 * variant[0] = values per lane of the fused z+y plane kernels (1, 2 or 4 for
 * 32-, 64- or 128-point planes; 0 = separate z and y passes), variant[1] =
 * values per lane of the warp-register X pass (0 = the shared-memory
 * Stockham X pass). */
int evpg_get_variant(void *ctx, int32_t variant[2]);
/* Device bytes evpg_create allocates for an n[0] x n[1] x n[2] RVE with
 * n_orient distinct orientations (for admission by HBM footprint); GND
 * densities add 193 bytes per voxel. */
int evpg_estimate_bytes(const int32_t n[3], int32_t precision, int32_t n_orient, int64_t *bytes);

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
 * first call on a device looks up that array's device address and writes the
 * twiddle tables of every axis length into it (a synchronous copy), so make
 * that first call outside any stream capture; later calls issue only memsets
 * and kernel launches on the given stream. Calls whose work overlaps on the GPU
 * share the array and race: serialise them. stream: a cudaStream_t or NULL. */
int evpg_green_correction_noalloc(const double *sig6, double *du9, int32_t n0, int32_t n1,
                                  int32_t n2, const double c0[81], const double s0[81],
                                  int32_t elast_bc, void *stream);

/* ---- batches: many RVE contexts advanced by the same launches ----
 * (no counterpart in the reference, which runs one RVE per MPI job)
 *
 * A batch holds up to any number of contexts of one precision and NR mode
 * ("slots"). evpg_batch_round runs one round on the batch's own stream: the
 * increment heads of the slots staged with evpg_batch_stage, then
 * equilibrium iterations -- each kernel launched once over all slots whose
 * loop is running -- with every slot's increment tail in the iteration where
 * its loop ends, until no slot is running or max_ticks iterations ran. A
 * slot that finished its increment in the round reads phase 3 (ended) from
 * evpg_batch_slot; one still iterating reads 2 and continues in the next
 * round. The round is one CUDA graph launch (conditional WHILE node),
 * re-captured when the slots change. A context belongs to at most one batch
 * at a time and issues no work of its own while the batch runs; results are
 * identical to the context's own evpg_increment. */
int evpg_batch_create(int32_t precision, int32_t nr_mode, void **batch_out);
int evpg_batch_destroy(void *batch);
/* Replace the slots (contexts stay owned by the caller). */
int evpg_batch_set(void *batch, void *const *ctxs, int32_t n);
/* Controls of slot's next increment (as evpg_increment). */
int evpg_batch_stage(void *batch, int32_t slot, const double udot_dt[3][3], int32_t creep,
                     const double disgrad_avg_actual[3][3], double time_tot, double e_vm,
                     int32_t tail);
int evpg_batch_round(void *batch, int32_t max_ticks, int32_t *ticks);
/* After a round: phase (0 idle, 1 staged, 2 running, 3 ended), sticky
 * status (evpg_status of the slot's last error) and the macro outputs of
 * the slot's current increment. Any out pointer may be NULL. */
int evpg_batch_slot(void *batch, int32_t slot, int32_t *phase, int32_t *status,
                    evpg_iter_out *it, evpg_incr_out *inc);
int evpg_batch_launch_count(void *batch, int64_t *n);
const char *evpg_batch_last_error(void);

/* ---- host driver: the reference's own input files and increment loop ---- */

/* GetNameList + SetupJob from the reference's namelist file; relative file
 * names inside it are resolved against the namelist's directory. rho0_path
 * (nullable) holds N doubles of initial SSD density, one per voxel, applied
 * to every slip system. precision: evpg_precision; nr_mode: evpg_nr_mode. */
int evpg_job_open(const char *input_path, const char *rho0_path, int32_t precision,
                  int32_t nr_mode, void **job_out);
/* evpg_job_open with options: EVPG_JOB_GND selects the first-order GND
 * densities (the reference built with DD_GND; L0 from the namelist). */
#define EVPG_JOB_GND 1
int evpg_job_open_opts(const char *input_path, const char *rho0_path, int32_t precision,
                       int32_t nr_mode, int32_t options, void **job_out);
int evpg_job_close(void *job);
void *evpg_job_ctx(void *job);
int evpg_job_nvox(void *job, int32_t n[3]);
int evpg_job_nsteps(void *job);

/* One increment of Evolution() (evolution.c:726-1520) on the device.
 * iters: equilibrium iterations taken. */
int evpg_job_increment(void *job, int32_t istep, int32_t *iters);

/* Batched increments of jobs (one precision and NR mode per batch):
 * evpg_job_stage puts increment istep of a job into a batch slot holding the
 * job's context; after evpg_batch_round, evpg_job_collect finishes the
 * job's increment if its slot ended (*ended = 1, iters = its equilibrium
 * iterations). evpg_jobs_run_batched runs nsteps[i] increments of every job
 * in one batch, rounds of at most max_ticks iterations, iters[i*stride+k]
 * = iterations of job i's increment k; results equal evpg_job_increment's. */
int evpg_job_stage(void *job, void *batch, int32_t slot, int32_t istep);
int evpg_job_collect(void *job, void *batch, int32_t slot, int32_t *ended, int32_t *iters);
int evpg_jobs_run_batched(void *const *jobs, int32_t n, const int32_t *nsteps, int32_t max_ticks,
                          int32_t *iters, int32_t stride, int64_t *rounds);

/* Mid-run load switch of a job (tension then shear, ...): the Voigt flags
 * and values of the velocity-gradient and stress boundary conditions
 * (VelGrad_BC_Flag, VelGrad_BC, Stress_BC_Flag, Stress_BC, init.c:865-901)
 * for the increments that follow; _from reads them from another namelist. */
int evpg_job_set_load(void *job, const int32_t velgrad_flag[6], const double velgrad[6],
                      const int32_t stress_flag[6], const double stress[6]);
int evpg_job_set_load_from(void *job, const char *input_path);
/* CellDim of a namelist file, without opening the job. */
int evpg_job_grid(const char *input_path, int32_t n[3]);

/* Scalars after the last increment: [0] TimeTot, [1] e_vm, [2] evmp,
 * [3] d_vm, [4] dvmp, [5] s_vm, [6] s_vm1, [7..15] SigAvg, [16..24] SigAvg1,
 * [25..32] rho averages as evpg_incr_out, [33] NR iterations of the
 * increment. */
int evpg_job_scalars(void *job, double *out, int32_t count);

/* Evolution() into outdir: vm.out, dd.out, err.out, iters.txt, and with
 * write_iout the reference's .iout dumps at PrintControl steps. nsteps < 0:
 * N_steps from the namelist. */
int evpg_job_run(void *job, const char *outdir, int32_t nsteps, int32_t write_iout);

/* ---- serving: continuous batching of solve requests ----
 * (no counterpart in the reference)
 *
 * Requests arrive at any time (evpg_server_submit: a namelist file, optional
 * per-voxel initial density, the number of increments and an optional load
 * switch to another namelist's boundary conditions after switch_step
 * increments). Loader threads open them in arrival order as soon as their
 * device footprint fits hbm_budget; the GPU thread admits opened requests
 * into free slots of one batch at every round boundary and advances all
 * slots together, round_ticks equilibrium iterations per round. Finished
 * solves release their device memory. Times are seconds since the server
 * was created. */
typedef struct evpg_server_cfg {
    int32_t precision, nr_mode;
    int64_t hbm_budget;    /* bytes of contexts the server may hold */
    int32_t max_slots;     /* RVEs advanced together */
    int32_t round_ticks;   /* equilibrium iterations per round */
    int32_t loaders;       /* host threads opening requests */
    int32_t keep_fields;   /* keep each finished solve's stress, SSD density and scalars */
    int32_t job_options;   /* evpg_job_open_opts options of every request (EVPG_JOB_GND) */
} evpg_server_cfg;

typedef struct evpg_request_info {
    int32_t state;         /* 0 queued, 1 loading, 2 ready, 3 running, 4 done, 5 failed */
    int32_t status;        /* evpg_status of a failed request */
    int32_t increments;    /* increments finished */
    int64_t iterations;    /* equilibrium iterations, summed over increments */
    double t_submit, t_admit, t_done;
    int64_t device_bytes;  /* footprint reserved while loaded */
} evpg_request_info;

typedef struct evpg_serve_stats {
    int32_t completed, failed;
    int64_t increments, iterations, rounds, ticks;
    double solve_p50, solve_p99;   /* submit -> done [s] */
    double incr_p50, incr_p99;     /* increment staged -> increment ended [s] */
    double span;                   /* first submit -> last completion [s] */
    double solves_per_s;
} evpg_serve_stats;

int evpg_server_create(const evpg_server_cfg *cfg, void **server_out);
int evpg_server_submit(void *server, const char *input_path, const char *rho0_path, int32_t nsteps,
                       int32_t switch_step, const char *switch_input_path, int64_t *id);
/* Wait until every submitted request finished (EVPG_ERR_ITERMAX on timeout). */
int evpg_server_wait(void *server, double timeout_s);
int evpg_server_request(void *server, int64_t id, evpg_request_info *info);
int evpg_server_stats(void *server, evpg_serve_stats *stats);
/* Kept results of a finished request (keep_fields): stress [nvox][6] in
 * .iout order, rho_s [nvox][12], the 34 scalars of evpg_job_scalars; any
 * output may be NULL. */
int evpg_server_result(void *server, int64_t id, double *sig6, double *rho_s, size_t nvox, double *scalars);
int evpg_server_destroy(void *server);

#ifdef __cplusplus
}
#endif
#endif
