/*
 * CPU restatement of SRX's EVP-FFT increment loop (TEST INFRASTRUCTURE ONLY).
 *
 * This is the oracle: the checker the GPU path is compared against, and the
 * timed CPU baseline. It restates, in plain C with the reference's order of
 * floating-point operations, the functions of the reference that the
 * equilibrium iteration runs (citations in evp_oracle.c). It is pinned
 * against the reference's own sources compiled with single-rank shims
 * (oracle/_ref, built by oracle/Makefile) through the fixtures under
 * tests/golden/. Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline legs may load it.
 */
#ifndef SRX_EVP_ORACLE_H
#define SRX_EVP_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct evo_job evo_job;

/* GetNameList + SetupJob (io.c:96-164, init.c:728-1216). File names inside
 * the namelist are resolved against the directory of `input_path`.
 * `rho0_path` (nullable): N doubles, per-voxel initial SSD density
 * (1e12 m^-2), applied to every slip system after set-up. Returns NULL and
 * fills `err` on failure. */
evo_job *evo_open(const char *input_path, const char *rho0_path, char *err, int errlen);
void evo_close(evo_job *j);

/* Worker threads for the per-voxel loops and FFT pencils (results are
 * bit-identical for any thread count). */
void evo_set_threads(int n);

int evo_nvox(const evo_job *j);

/* 0: plain NR (evolution.c:372-377, the top-level build); 1: NR_MODIFIED
 * backtracking line search (evolution.c:280-371, on in the FFTW3 variant,
 * fftw3version-NOSMOOTHING/evpFlags.h:21). */
void evo_set_nr_mode(evo_job *j, int mode);
int evo_nsteps(const evo_job *j);

/* First-order GND densities (the reference built with DD_GND, which implies
 * DD_GND_FIRST_ORDER, evpFlags.h:29-32): slip-rate gradients with grain-
 * boundary stencils (constitutive.c:731-1112), GND rates in the dislocation
 * update (constitutive.c:1428-1522), their projections in the flow rule
 * (constitutive.c:558-577) and rho_tot (evolution.c:1041-1045). Set before
 * the first increment; off by default (the shipped configuration). */
void evo_set_gnd(evo_job *j, int on);

/* One increment of Evolution() (evolution.c:726-1520) without file output.
 * Returns 0, or a nonzero status: 1 NaN in the flow rule, 2 singular LU. */
int evo_increment(evo_job *j, int istep, int *iters);

/* Whole Evolution() into `outdir`: vm.out, dd.out, err.out, iters.txt
 * (one line per increment: istep iterations) and errors.txt (the per-iteration
 * lines the reference prints, evolution.c:1254-1255); with write_iout the
 * reference's .iout dumps at PrintControl steps (io.c:322-995; the
 * new_position record is written as zeros). nsteps < 0 means N_steps. */
int evo_run(evo_job *j, const char *outdir, int nsteps, int write_iout);

/* Raw pointers into the AoS state (reference layout, evp.h:429-456):
 * "Sig","DisGrad","Eps","Edot","VelGrad","TranMat" ([N][3][3]);
 * "rho_s","rho_m","rho_F","rho_P","gamdot","gam_acum","trial_gam_acum",
 * "rho_dipole","rho_forest","rho_inplane","rho_g1","rho_g2" ([N][12]); "rho_tot" ([N]);
 * "Schm_gr" ([N][12][5]); set-up arrays "C066","S066" (6x6), "S0" (3^4),
 * "Chi","Chi_1" ([2][12][12]), "Shear_G" ([2]), "bb_B" ([2][12]),
 * "Schm_xt" ([2][12][5]); "scalars" (see evp_oracle.c). */
double *evo_field(evo_job *j, const char *name);

/* Building blocks, for unit parity of single stages. */
void evo_update_schmid(evo_job *j);                          /* kinematics.c:430-463 */
int evo_update_stress(evo_job *j, double *err_e, double *err_s); /* evolution.c:157-427 */
void evo_get_smacro(evo_job *j);                             /* evolution.c:590-664 */
void evo_spectral(evo_job *j);                               /* evolution.c:1157-1201 */
void evo_begin(evo_job *j);      /* increment head, evolution.c:1030-1141 */
int evo_iteration(evo_job *j);   /* one pass of the loop body, evolution.c:1151-1257 */

#ifdef __cplusplus
}
#endif
#endif
