/*
 * CPU restatement of SRX's EVP-FFT increment loop (TEST INFRASTRUCTURE ONLY;
 * see evp_oracle.h). Every function cites the reference lines it restates.
 * Floating-point expressions keep the reference's association order so that
 * results match the reference compiled with the same CPU FFT bit for bit;
 * build with -ffp-contract=off.
 *
 * Deliberate differences, none of which changes a result:
 *  - C_gr and its inverse are computed once per distinct (Euler angles,
 *    phase) instead of once per voxel / per NR call (pure functions of the
 *    same inputs, so the bits are identical);
 *  - the Green operator is evaluated per frequency inside the contraction
 *    instead of being stored (init.c:542-592 restated in place);
 *  - error and average sums are accumulated into per-voxel slots and summed
 *    serially in voxel order, which equals the reference's serial order for
 *    any thread count;
 *  - with GND densities on (evo_set_gnd, the reference's DD_GND with
 *    DD_GND_FIRST_ORDER) the slip-rate gradient of each voxel is formed where
 *    the densities are updated, from the neighbours' shear rates, instead of
 *    in a separate pass over all voxels (Gradient_ShearRate,
 *    constitutive.c:881-1112): the shear rates are not changed in between;
 *  - the displacement post-step (evolution.c:1401-1425) is restated by what
 *    it computes as written: its per-frequency sums go into scalars and one
 *    element past fft_data, so the inverse transform acts on the forward
 *    transform of fluctuation[:][mi][2], and displacement_fluct[mi] is minus
 *    the round trip of that component.
 */
#include "evp_oracle.h"
#include "fft_cpu.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NPH 2
#define NS 12

/* evp.h:84-94 */
#define R_PI 3.14159265359
#define R_TWO_PI 6.28318530718
#define TRIAL_FREQ_DRX 1.0E10
#define EV_IN_J 1.60217733e-19
#define MY_J_IN_EV 0.62415063631
#define BOLZ 1.380658e-23
#define EPSILON_STRESS 1.0E-4 /* evp.h:21 EPSILON */
#define EPSILON_FFT 1E-5
#define SRX_MAX(x, y) ((x) > (y) ? (x) : (y)) /* V3math.h:7 */

typedef double t2[3][3];
typedef double v66[6][6];
typedef double t4[3][3][3][3];

static int g_threads = 1;
void evo_set_threads(int n) { g_threads = n > 0 ? n : 1; }

/* ------------------------------------------------------------ namelist */

typedef struct {
    int CellDim[3], N_phases, Type_phases[2], N_steps, Update_Flag, Hard_Flag, Tex_Flag;
    int IterMax, PrintControl[2], VelGrad_BC_Flag[6], Stress_BC_Flag[6], ElastBC;
    int nucleus_radius, CellDim_pf[3], RandSeed, Nucl_Static_Flag;
    double TimeStep, Err, VelGrad_BC[6], Stress_BC[6], ElastConst_PhaseI[4],
        ElastConst_PhaseII[4];
    char Slip_PhaseI[100], Slip_PhaseII[100], initial_ms[100];
    double a0[2], L0, GND_ScaleRatio, T__K, Q_slip[2], Q_bulk[2], C_1[2], C_2[2], C_3[2],
        C_4[2], C_5[2], C_6[2], C_7[2], C_8[2], Selfinter0[2], Coplanar0[2], CrossSlip0[2],
        GlissileJunction0[2], HirthLock0[2], LomerCottrellLock0[2], rho_SSD_initial, D_0;
    double E_gb, M_gb, Scale_Fdeform, k_c, alpha, zeta_kc, age_drx, ssdScaler_DRX,
        gndScaler_DRX, sigScaler_DRX, tau_DRX, DeltaQ_DRX, DeltaTau_DRX, pf_length_scale,
        pf_time_step;
} namelist;

enum { NI, NR, NSTR };
typedef struct { const char *name; void *ptr; int type, len, status; } nlent;

/* GetNameList(), io.c:96-164: first definition wins, a blank-but-not-empty
 * line stops parsing, a last line without newline is dropped. */
static int read_namelist(const char *path, namelist *nl)
{
    nlent t[] = {
        {"CellDim", nl->CellDim, NI, 3}, {"N_phases", &nl->N_phases, NI, 1},
        {"Type_phases", nl->Type_phases, NI, 2}, {"TimeStep", &nl->TimeStep, NR, 1},
        {"N_steps", &nl->N_steps, NI, 1}, {"Update_Flag", &nl->Update_Flag, NI, 1},
        {"Hard_Flag", &nl->Hard_Flag, NI, 1}, {"Tex_Flag", &nl->Tex_Flag, NI, 1},
        {"IterMax", &nl->IterMax, NI, 1}, {"PrintControl", nl->PrintControl, NI, 2},
        {"Err", &nl->Err, NR, 1}, {"VelGrad_BC_Flag", nl->VelGrad_BC_Flag, NI, 6},
        {"VelGrad_BC", nl->VelGrad_BC, NR, 6}, {"Stress_BC_Flag", nl->Stress_BC_Flag, NI, 6},
        {"Stress_BC", nl->Stress_BC, NR, 6}, {"ElastBC", &nl->ElastBC, NI, 1},
        {"ElastConst_PhaseI", nl->ElastConst_PhaseI, NR, 4},
        {"ElastConst_PhaseII", nl->ElastConst_PhaseII, NR, 4},
        {"Slip_PhaseI", nl->Slip_PhaseI, NSTR, 1}, {"Slip_PhaseII", nl->Slip_PhaseII, NSTR, 1},
        {"initial_ms", nl->initial_ms, NSTR, 1}, {"a0", nl->a0, NR, 2}, {"L0", &nl->L0, NR, 1},
        {"GND_ScaleRatio", &nl->GND_ScaleRatio, NR, 1}, {"T__K", &nl->T__K, NR, 1},
        {"Q_slip", nl->Q_slip, NR, 2}, {"Q_bulk", nl->Q_bulk, NR, 2}, {"C_1", nl->C_1, NR, 2},
        {"C_2", nl->C_2, NR, 2}, {"C_3", nl->C_3, NR, 2}, {"C_4", nl->C_4, NR, 2},
        {"C_5", nl->C_5, NR, 2}, {"C_6", nl->C_6, NR, 2}, {"C_7", nl->C_7, NR, 2},
        {"C_8", nl->C_8, NR, 2}, {"Selfinter0", nl->Selfinter0, NR, 2},
        {"Coplanar0", nl->Coplanar0, NR, 2}, {"CrossSlip0", nl->CrossSlip0, NR, 2},
        {"GlissileJunction0", nl->GlissileJunction0, NR, 2},
        {"HirthLock0", nl->HirthLock0, NR, 2},
        {"LomerCottrellLock0", nl->LomerCottrellLock0, NR, 2},
        {"rho_SSD_initial", &nl->rho_SSD_initial, NR, 1}, {"D_0", &nl->D_0, NR, 1},
        {"nucleus_radius", &nl->nucleus_radius, NI, 1}, {"CellDim_pf", nl->CellDim_pf, NI, 3},
        {"RandSeed", &nl->RandSeed, NI, 1}, {"E_gb", &nl->E_gb, NR, 1},
        {"M_gb", &nl->M_gb, NR, 1}, {"Scale_Fdeform", &nl->Scale_Fdeform, NR, 1},
        {"k_c", &nl->k_c, NR, 1}, {"Nucl_Static_Flag", &nl->Nucl_Static_Flag, NI, 1},
        {"alpha", &nl->alpha, NR, 1}, {"zeta_kc", &nl->zeta_kc, NR, 1},
        {"age_drx", &nl->age_drx, NR, 1}, {"ssdScaler_DRX", &nl->ssdScaler_DRX, NR, 1},
        {"gndScaler_DRX", &nl->gndScaler_DRX, NR, 1},
        {"sigScaler_DRX", &nl->sigScaler_DRX, NR, 1}, {"tau_DRX", &nl->tau_DRX, NR, 1},
        {"DeltaQ_DRX", &nl->DeltaQ_DRX, NR, 1}, {"DeltaTau_DRX", &nl->DeltaTau_DRX, NR, 1},
        {"pf_length_scale", &nl->pf_length_scale, NR, 1},
        {"pf_time_step", &nl->pf_time_step, NR, 1},
    };
    const int nt = (int)(sizeof t / sizeof t[0]);
    char buff[200], *tok;
    FILE *fp = fopen(path, "r");
    int k, j;
    if (!fp) return -1;
    memset(nl, 0, sizeof *nl);
    for (;;) {
        if (!fgets(buff, 200, fp)) break;
        if (feof(fp)) break;
        if (buff[0] == '#' || buff[0] == '\n') continue;
        tok = strtok(buff, " \t\n");
        if (!tok) break;
        for (k = 0; k < nt; k++) {
            if (strcmp(tok, t[k].name) != 0) continue;
            if (t[k].status == 0) {
                t[k].status = 1;
                for (j = 0; j < t[k].len; j++) {
                    tok = strtok(NULL, ", \t\n");
                    if (!tok) { t[k].status = 2; continue; }
                    if (t[k].type == NI) ((int *)t[k].ptr)[j] = (int)atol(tok);
                    else if (t[k].type == NR) ((double *)t[k].ptr)[j] = atof(tok);
                    else strcpy((char *)t[k].ptr + j, tok);
                }
            }
            break;
        }
    }
    fclose(fp);
    return 0;
}

/* ------------------------------------------------------------- the job */

struct evo_job {
    namelist nl;
    int n0, n1, n2, N;
    double WGT, Wgt_ph1;
    double B[6][3][3];
    int nSYS[NPH];
    double tau0[NPH];                 /* tau[jph][0][0] (constitutive.c:537) */
    double bn[NPH][NS][3], bb[NPH][NS][3], bb_B[NPH][NS];
    double Schm_xt[NPH][NS][5];
    double Shear_G[NPH];
    double Cijkl[NPH][3][3][3][3];
    double Chi[NPH][NS][NS], Chi_1[NPH][NS][NS];
    v66 C066, S066;
    t4 C0, S0;
    t2 Udot, Udot_s, Udot_a, Scauchy;
    int CREEP_FLAG;
    double d_vm, e_vm, s_vm, s_vm1, TimeTot, Err_e, Err_s;
    t2 DisGradAvg, dDisGradAvg, dDisGradAvg_acum, SigAvg, SigAvg1, SigDevAvg, EpsAvg, EdotAvg,
        VelGradAvg, DisGradAvg_t, DisGradAvg_actual;
    double evmp, dvmp;
    double rho_avg[8]; /* F, P, s, m, g, dipole, forest, inplane (constitutive.c:1681-1808) */
    /* per voxel */
    int *grain_f, *phase_f, *oid;
    int n_orient;
    v66 *Cg, *Sg;         /* per distinct orientation */
    double *orient_key;   /* 4 per orientation: ph, th, om, jph */
    t2 *Sig, *DisGrad, *Eps, *Edot, *VelGrad, *TranMat, *fluct;
    double (*disp)[3];    /* displacement_fluct */
    double (*Schm_gr)[NS][5];
    double (*rho_s)[NS], (*rho_m)[NS], (*rho_F)[NS], (*rho_P)[NS], (*gamdot)[NS],
        (*gam_acum)[NS], (*trial_gam_acum)[NS], (*rho_dipole)[NS], (*rho_forest)[NS],
        (*rho_inplane)[NS], (*rho_dot_s)[NS];
    double *rho_tot;
    /* first-order GND densities (DD_GND): rho_g1 screw, rho_g2 edge type I; the
     * edge type II density stays zero to first order (constitutive.c:1494-1518) */
    int gnd;
    double (*rho_g1)[NS], (*rho_g2)[NS];
    unsigned char *gb;    /* same-grain neighbour bits, see gb_masks() */
    double bp[NPH][NS][3];                       /* b x n, init.c:198-203 */
    double cos_g1[NPH][NS][NS], sin_g1[NPH][NS][NS], cos_g2[NPH][NS][NS], sin_g2[NPH][NS][NS];
    double *kr, *ki;      /* kSig_r/kSig_i, [N][9] */
    double *fft;          /* N complex */
    double *vox_e, *vox_s;
    int *vox_flag;
    double scalars[32];
    int status;
    int nr_mode; /* 0 plain NR, 1 NR_MODIFIED line search */
};

int evo_nvox(const evo_job *j) { return j->N; }
void evo_set_nr_mode(evo_job *j, int mode) { j->nr_mode = mode; }
int evo_nsteps(const evo_job *j) { return j->nl.N_steps; }

/* ------------------------------------------------------------- algebra */

/* chg_basis(opt=0), kinematics.c:28-54 */
static void make_B(double B[6][3][3])
{
    const double RSQ2 = 0.70710678118654744, RSQ3 = 0.57735026918962584,
                 RSQ6 = 0.40824829046386304;
    memset(B, 0, sizeof(double) * 54);
    B[1][0][0] = -1. * RSQ6; B[1][1][1] = -1. * RSQ6; B[1][2][2] = 2. * RSQ6;
    B[0][0][0] = -1. * RSQ2; B[0][1][1] = RSQ2;
    B[2][1][2] = RSQ2; B[2][2][1] = RSQ2;
    B[3][0][2] = RSQ2; B[3][2][0] = RSQ2;
    B[4][0][1] = RSQ2; B[4][1][0] = RSQ2;
    B[5][0][0] = RSQ3; B[5][1][1] = RSQ3; B[5][2][2] = RSQ3;
}

/* chg_basis opt 2 / chg_basis5 opt 2 (kinematics.c:62-69,143-150) */
static void t2_to_v(const double B[6][3][3], const t2 T, double *V, int n)
{
    int i, a, b;
    for (i = 0; i < n; i++) {
        V[i] = 0.0;
        for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) V[i] += T[a][b] * B[i][a][b];
    }
}

/* chg_basis opt 1 / chg_basis5 opt 1 (kinematics.c:55-61,136-142) */
static void v_to_t2(const double B[6][3][3], const double *V, t2 T, int n)
{
    int i, a, b;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            T[a][b] = 0.0;
            for (i = 0; i < n; i++) T[a][b] += V[i] * B[i][a][b];
        }
}

/* chg_basis opt 3 (kinematics.c:70-77) */
static void c66_to_t4(const double B[6][3][3], const v66 C, t4 T)
{
    int a, b, c, d, i, k;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++)
            for (c = 0; c < 3; c++)
                for (d = 0; d < 3; d++) {
                    T[a][b][c][d] = 0.0;
                    for (i = 0; i < 6; i++)
                        for (k = 0; k < 6; k++) T[a][b][c][d] += C[i][k] * B[i][a][b] * B[k][c][d];
                }
}

/* chg_basis opt 4 (kinematics.c:78-87) */
static void t4_to_c66(const double B[6][3][3], const t4 T, v66 C)
{
    int a, b, c, d, i, k;
    for (i = 0; i < 6; i++)
        for (k = 0; k < 6; k++) {
            C[i][k] = 0.0;
            for (a = 0; a < 3; a++)
                for (b = 0; b < 3; b++)
                    for (c = 0; c < 3; c++)
                        for (d = 0; d < 3; d++) C[i][k] += T[a][b][c][d] * B[i][a][b] * B[k][c][d];
        }
}

/* LU_dcmp + LU_bksb + LU_inv_66, kinematics.c:282-428 (Numerical Recipes
 * Crout with implicit scaling; pivot floor 1e-5 -> 1e-20; forward
 * substitution starts at the first entry above 1e-5). Returns 1 when a row
 * is all below 1e-5 (the reference exits with status 35). */
static int lu_inv66(v66 c)
{
    int indx[6], i, imax = 0, j, k, ii, ip, n = 6;
    double big, dum, sum, temp, vv[6], col[6], y[6][6];
    for (i = 0; i < n; i++) {
        big = 0.0;
        for (j = 0; j < n; j++)
            if ((temp = fabs(c[i][j])) > big) big = temp;
        if (fabs(big) < EPSILON_FFT) return 1;
        vv[i] = 1.0 / big;
    }
    for (j = 0; j < n; j++) {
        for (i = 0; i < j; i++) {
            sum = c[i][j];
            for (k = 0; k < i; k++) sum -= c[i][k] * c[k][j];
            c[i][j] = sum;
        }
        big = 0.0;
        for (i = j; i < n; i++) {
            sum = c[i][j];
            for (k = 0; k < j; k++) sum -= c[i][k] * c[k][j];
            c[i][j] = sum;
            if ((dum = vv[i] * fabs(sum)) >= big) {
                big = dum;
                imax = i;
            }
        }
        if (j != imax) {
            for (k = 0; k < n; k++) {
                dum = c[imax][k];
                c[imax][k] = c[j][k];
                c[j][k] = dum;
            }
            vv[imax] = vv[j];
        }
        indx[j] = imax;
        if (fabs(c[j][j]) < 1E-5) c[j][j] = 1.0E-20;
        if (j != n - 1) {
            dum = 1.0 / (c[j][j]);
            for (i = j + 1; i < n; i++) c[i][j] *= dum;
        }
    }
    for (k = 0; k < n; k++) {
        for (i = 0; i < n; i++) col[i] = 0.0;
        col[k] = 1.0;
        ii = -1;
        for (i = 0; i < n; i++) {
            ip = indx[i];
            sum = col[ip];
            col[ip] = col[i];
            if (ii >= 0)
                for (j = ii; j <= i - 1; j++) sum -= c[i][j] * col[j];
            else if (fabs(sum) > 1E-5)
                ii = i;
            col[i] = sum;
        }
        for (i = n - 1; i >= 0; i--) {
            sum = col[i];
            for (j = i + 1; j < n; j++) sum -= c[i][j] * col[j];
            col[i] = sum / c[i][i];
        }
        for (i = 0; i < n; i++) y[i][k] = col[i];
    }
    memcpy(c, y, sizeof(v66));
    return 0;
}

/* EulerToTransMatrix opt 2, kinematics.c:218-234 (Bunge, radians) */
static void euler_to_a(double t1, double ph, double t2v, t2 a)
{
    double ct1 = cos(t1), st1 = sin(t1), cph = cos(ph), sph = sin(ph), ct2 = cos(t2v),
           st2 = sin(t2v);
    a[0][0] = ct1 * ct2 - st1 * st2 * cph;
    a[0][1] = st1 * ct2 + ct1 * st2 * cph;
    a[0][2] = st2 * sph;
    a[1][0] = -1.0 * ct1 * st2 - st1 * ct2 * cph;
    a[1][1] = -1.0 * st1 * st2 + ct1 * ct2 * cph;
    a[1][2] = ct2 * sph;
    a[2][0] = st1 * sph;
    a[2][1] = -1.0 * ct1 * sph;
    a[2][2] = cph;
}

/* EulerToTransMatrix opt 1, kinematics.c:198-217 (degrees out) */
static void a_to_euler(const t2 a, double *t1, double *ph, double *t2v)
{
    double p = acos(a[2][2]), x1, x2, sph;
    if (fabs(a[2][2]) > 0.9999) {
        x2 = 0.;
        x1 = atan2(a[0][1], a[0][0]);
    } else {
        sph = sin(p);
        x1 = atan2(a[2][0] / sph, -1.0 * a[2][1] / sph);
        x2 = atan2(a[0][2] / sph, a[1][2] / sph);
    }
    *ph = p * (180. / R_PI);
    *t1 = x1 * (180. / R_PI);
    *t2v = x2 * (180. / R_PI);
}

/* VonMises, kinematics.c:465-483 */
static double von_mises(const t2 t)
{
    double trace = t[0][0] + t[1][1] + t[2][2], dt, vm = 0.0;
    int a, b;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            dt = (t[a][b] + t[b][a]) / 2. - (double)(a == b) * trace / 3.0;
            vm += dt * dt;
        }
    return sqrt(2. / 3. * vm);
}

/* ElastStiffnessMatrix, init.c:10-50 (cubic) */
static void cubic_C(const double *ec, t4 c)
{
    int i, j, k, l;
    memset(c, 0, sizeof(t4));
    for (i = 0; i < 3; i++) c[i][i][i][i] = ec[0];
    for (i = 0; i < 3; i++)
        for (j = 0; j < 3; j++)
            if (i != j) {
                c[i][i][j][j] = ec[1];
                c[i][j][i][j] = ec[2];
                c[i][j][j][i] = ec[2];
            }
    (void)k; (void)l;
}

/* InteractionStrengthMatrix, init.c:594-703 (FCC, Arsenlis & Parks labels) */
static void interaction(double self, double copl, double cross, double gliss, double hirth,
                        double lomer, double chi[NS][NS])
{
    /* 0 self, 1 coplanar, 2 cross, 3 glissile, 4 hirth, 5 lomer */
    static const char L[NS][NS + 1] = {
        "011435233453", "001323345543", "000534354332", "000011453233",
        "000001543345", "000000332354", "000000011435", "000000001323",
        "000000000534", "000000000011", "000000000001", "000000000000",
    };
    const double v[6] = {self, copl, cross, gliss, hirth, lomer};
    int i, j;
    for (i = 0; i < NS; i++)
        for (j = i; j < NS; j++) chi[i][j] = (i == j) ? self : v[L[i][j] - '0'];
    for (i = 1; i < NS; i++)
        for (j = 0; j < i; j++) chi[i][j] = chi[j][i];
}

/* --------------------------------------------------------------- set-up */

static void set_err(char *err, int n, const char *msg, const char *arg)
{
    if (err && n > 0) snprintf(err, (size_t)n, "%s%s", msg, arg ? arg : "");
}

static void resolve(const char *input_path, const char *name, char *out, size_t n)
{
    const char *slash = strrchr(input_path, '/');
    if (name[0] == '/' || !slash) {
        snprintf(out, n, "%s", name);
    } else {
        snprintf(out, n, "%.*s/%s", (int)(slash - input_path), input_path, name);
    }
}

/* PlasticInit, init.c:52-231 */
static int plastic_init(evo_job *j, const char *path, int phase)
{
    FILE *fp = fopen(path, "r");
    char buf[80] = {0}, xs[16];
    int i, k, mx, m_count = 0, nmodes_max = 0, nmodes = 0, imode[16], nsmx = 0, isectwx;
    double ax[3], nrsx, gamd0x, twshx, tau0xf = 0, tau0xb, tau1x, thet0, thet1, hs, hl, norm;
    if (!fp) return -1;
#define RD() (void)!fgets(buf, 80, fp)
    RD(); RD(); sscanf(buf, "%15s", xs);
    RD(); RD(); RD(); sscanf(buf, "%lf %lf %lf", &ax[0], &ax[1], &ax[2]);
    RD(); RD(); RD(); sscanf(buf, "%d", &nmodes_max);
    RD(); RD(); RD(); sscanf(buf, "%d", &nmodes);
    if (nmodes < 1 || nmodes > 16) { fclose(fp); return -2; }
    RD(); RD();
    for (i = 0; i < nmodes; i++) { RD(); sscanf(buf, "%d", &imode[i]); }
    RD();
    for (i = 0; i < nmodes_max; i++) {
        int match = 0;
        RD(); sscanf(buf, "%*s %*s %d %*s", &mx);
        for (k = 0; k < nmodes; k++) if (mx == imode[k]) { match = 1; m_count++; break; }
        RD(); RD();
        sscanf(buf, "%d %lf %lf %lf %d", &nsmx, &nrsx, &gamd0x, &twshx, &isectwx);
        RD(); RD();
        sscanf(buf, "%lf %lf %lf %lf %lf", &tau0xf, &tau0xb, &tau1x, &thet0, &thet1);
        RD(); RD(); sscanf(buf, "%lf %lf", &hs, &hl);
        RD();
        if (match) {
            if (nsmx > NS || nsmx < 1) { fclose(fp); return -3; }
            j->nSYS[phase] = nsmx;
            j->tau0[phase] = tau0xf;
            for (k = 0; k < nsmx; k++) {
                RD();
                sscanf(buf, "%lf %lf %lf %lf %lf %lf", &j->bn[phase][k][0], &j->bn[phase][k][1],
                       &j->bn[phase][k][2], &j->bb[phase][k][0], &j->bb[phase][k][1],
                       &j->bb[phase][k][2]);
            }
        } else {
            for (k = 0; k < nsmx; k++) RD();
        }
    }
#undef RD
    fclose(fp);
    for (i = 0; i < nmodes; i++) {
        for (k = 0; k < j->nSYS[phase]; k++) {
            t2 aux;
            double a5[6];
            int a, b;
            norm = sqrt(pow(j->bn[phase][k][0], 2.0) + pow(j->bn[phase][k][1], 2.0) +
                        pow(j->bn[phase][k][2], 2.0));
            for (mx = 0; mx < 3; mx++) j->bn[phase][k][mx] /= norm;
            norm = sqrt(pow(j->bb[phase][k][0], 2.0) + pow(j->bb[phase][k][1], 2.0) +
                        pow(j->bb[phase][k][2], 2.0));
            j->bb_B[phase][k] = j->nl.a0[phase] / sqrt(2.0);
            for (mx = 0; mx < 3; mx++) j->bb[phase][k][mx] /= norm;
            norm = 0.0;
            for (mx = 0; mx < 3; mx++) norm += j->bn[phase][k][mx] * j->bb[phase][k][mx];
            if (norm > 1E-3) return -4;
            /* sense vector p = b x n, init.c:198-203 */
            j->bp[phase][k][0] = j->bb[phase][k][1] * j->bn[phase][k][2] - j->bb[phase][k][2] * j->bn[phase][k][1];
            j->bp[phase][k][1] = j->bb[phase][k][2] * j->bn[phase][k][0] - j->bb[phase][k][0] * j->bn[phase][k][2];
            j->bp[phase][k][2] = j->bb[phase][k][0] * j->bn[phase][k][1] - j->bb[phase][k][1] * j->bn[phase][k][0];
            for (a = 0; a < 3; a++)
                for (b = 0; b < 3; b++)
                    aux[a][b] = (j->bn[phase][k][a] * j->bb[phase][k][b] +
                                 j->bn[phase][k][b] * j->bb[phase][k][a]) / 2.0;
            t2_to_v(j->B, aux, a5, 5);
            for (mx = 0; mx < 5; mx++) j->Schm_xt[phase][k][mx] = a5[mx];
        }
    }
    (void)m_count;
    return 0;
}

#define ALLOC(p, n) ((p) = calloc((size_t)(n), sizeof(*(p))))

static int alloc_fields(evo_job *j)
{
    const int N = j->N;
    int ok = 1;
    ok &= ALLOC(j->grain_f, N) != 0; ok &= ALLOC(j->phase_f, N) != 0; ok &= ALLOC(j->oid, N) != 0;
    ok &= ALLOC(j->Sig, N) != 0; ok &= ALLOC(j->DisGrad, N) != 0; ok &= ALLOC(j->Eps, N) != 0;
    ok &= ALLOC(j->Edot, N) != 0; ok &= ALLOC(j->VelGrad, N) != 0;
    ok &= ALLOC(j->TranMat, N) != 0; ok &= ALLOC(j->fluct, N) != 0; ok &= ALLOC(j->disp, N) != 0;
    ok &= ALLOC(j->Schm_gr, N) != 0;
    ok &= ALLOC(j->rho_s, N) != 0; ok &= ALLOC(j->rho_m, N) != 0; ok &= ALLOC(j->rho_F, N) != 0;
    ok &= ALLOC(j->rho_P, N) != 0; ok &= ALLOC(j->gamdot, N) != 0;
    ok &= ALLOC(j->gam_acum, N) != 0; ok &= ALLOC(j->trial_gam_acum, N) != 0;
    ok &= ALLOC(j->rho_dipole, N) != 0; ok &= ALLOC(j->rho_forest, N) != 0;
    ok &= ALLOC(j->rho_inplane, N) != 0; ok &= ALLOC(j->rho_dot_s, N) != 0;
    ok &= ALLOC(j->rho_tot, N) != 0;
    ok &= ALLOC(j->rho_g1, N) != 0; ok &= ALLOC(j->rho_g2, N) != 0; ok &= ALLOC(j->gb, N) != 0;
    ok &= ALLOC(j->kr, 9 * (size_t)N) != 0; ok &= ALLOC(j->ki, 9 * (size_t)N) != 0;
    ok &= ALLOC(j->fft, 2 * (size_t)N) != 0;
    ok &= ALLOC(j->vox_e, N) != 0; ok &= ALLOC(j->vox_s, N) != 0; ok &= ALLOC(j->vox_flag, N) != 0;
    return ok ? 0 : -1;
}

/* InitMicroStruct, init.c:233-396 */
static int init_microstructure(evo_job *j, const char *path)
{
    FILE *fp = fopen(path, "r");
    char buf[80] = {0};
    int v, cap = 64, nph1 = 0, a, b;
    v66 c066 = {{0}};
    if (!fp) return -1;
    j->n_orient = 0;
    j->orient_key = malloc(sizeof(double) * 4 * (size_t)cap);
    j->Cg = malloc(sizeof(v66) * (size_t)cap);
    j->Sg = malloc(sizeof(v66) * (size_t)cap);
    for (v = 0; v < j->N; v++) {
        double ph = 0, th = 0, om = 0;
        int ii = 0, jj = 0, kk = 0, jgr = 0, jph = 0, idx, o;
        if (!fgets(buf, 80, fp)) { fclose(fp); return -2; }
        sscanf(buf, "%lf %lf %lf %d %d %d %d %d", &ph, &th, &om, &ii, &jj, &kk, &jgr, &jph);
        idx = ((ii - 1) * j->n1 + jj - 1) * j->n2 + kk - 1;
        if (idx != v) { fclose(fp); return -3; }
        if (jph < 1 || jph > NPH) { fclose(fp); return -4; }
        if (jph == 1) nph1++;
        j->grain_f[v] = jgr;
        j->phase_f[v] = jph;
        j->oid[v] = -1;
        if (!j->nl.Type_phases[jph - 1]) {
            t2 sa2xt;
            ph *= R_PI / 180.; th *= R_PI / 180.; om *= R_PI / 180.;
            euler_to_a(ph, th, om, sa2xt);
            for (a = 0; a < 3; a++)
                for (b = 0; b < 3; b++) j->TranMat[v][a][b] = sa2xt[b][a];
            for (o = 0; o < j->n_orient; o++) {
                const double *kk4 = j->orient_key + 4 * o;
                if (kk4[0] == ph && kk4[1] == th && kk4[2] == om && kk4[3] == (double)jph) break;
            }
            if (o == j->n_orient) {
                t4 caux;
                int p, q, r, s, m, n, pp, qq;
                if (j->n_orient == cap) {
                    cap *= 2;
                    j->orient_key = realloc(j->orient_key, sizeof(double) * 4 * (size_t)cap);
                    j->Cg = realloc(j->Cg, sizeof(v66) * (size_t)cap);
                    j->Sg = realloc(j->Sg, sizeof(v66) * (size_t)cap);
                }
                /* Ten4thTransform opt 2, kinematics.c:262-274 */
                for (p = 0; p < 3; p++)
                    for (q = 0; q < 3; q++)
                        for (r = 0; r < 3; r++)
                            for (s = 0; s < 3; s++) {
                                caux[p][q][r][s] = 0.0;
                                for (m = 0; m < 3; m++)
                                    for (n = 0; n < 3; n++)
                                        for (pp = 0; pp < 3; pp++)
                                            for (qq = 0; qq < 3; qq++)
                                                caux[p][q][r][s] += sa2xt[m][p] * sa2xt[n][q] *
                                                                    sa2xt[pp][r] * sa2xt[qq][s] *
                                                                    j->Cijkl[jph - 1][m][n][pp][qq];
                            }
                t4_to_c66(j->B, caux, j->Cg[o]);
                memcpy(j->Sg[o], j->Cg[o], sizeof(v66));
                if (lu_inv66(j->Sg[o])) { fclose(fp); return -5; }
                j->orient_key[4 * o] = ph;
                j->orient_key[4 * o + 1] = th;
                j->orient_key[4 * o + 2] = om;
                j->orient_key[4 * o + 3] = (double)jph;
                j->n_orient++;
            }
            j->oid[v] = o;
            for (a = 0; a < 6; a++)
                for (b = 0; b < 6; b++) c066[a][b] += j->Cg[o][a][b];
        }
    }
    fclose(fp);
    j->Wgt_ph1 = (1.0 * (double)nph1) / j->N;
    for (a = 0; a < 6; a++)
        for (b = 0; b < 6; b++) {
            j->C066[a][b] = c066[a][b];
            j->C066[a][b] *= j->WGT;
        }
    memcpy(j->S066, j->C066, sizeof(v66));
    if (lu_inv66(j->S066)) return -6;
    c66_to_t4(j->B, j->C066, j->C0);
    c66_to_t4(j->B, j->S066, j->S0);
    return 0;
}

static void voigt_to_full(const double *v, t2 m)
{
    m[0][0] = v[0]; m[0][1] = v[5]; m[0][2] = v[4];
    m[1][0] = v[5]; m[1][1] = v[1]; m[1][2] = v[3];
    m[2][0] = v[4]; m[2][1] = v[3]; m[2][2] = v[2];
}

static double shear_modulus(const double *ec)
{
    /* init.c:827 */
    return 0.1 * (ec[0] - ec[1] + 3 * ec[2]) +
           (0.5) * (5 * (ec[0] - ec[1]) * ec[2]) / (4 * ec[2] + 3 * (ec[0] - ec[1]));
}

/* Gradient_ExchangeGrainID, constitutive.c:731-879, on one rank (periodic
 * neighbours): bit 0/1 x+/x- neighbour in the same grain, 2/3 y+/y-, 4 z+,
 * 5 the "z-" check, which compares with the y- neighbour as the reference
 * does (GB_checkZ[pIDX][1], constitutive.c:821, 842, 859). */
static void gb_masks(evo_job *j)
{
    const int n0 = j->n0, n1 = j->n1, n2 = j->n2;
    int x, y, z;
    for (x = 0; x < n0; x++)
        for (y = 0; y < n1; y++)
            for (z = 0; z < n2; z++) {
                const int xp = (x + 1) % n0, xm = (x + n0 - 1) % n0, yp = (y + 1) % n1,
                          ym = (y + n1 - 1) % n1, zp = (z + 1) % n2;
                const int v = (x * n1 + y) * n2 + z, g = j->grain_f[v];
                unsigned char m = 0;
                m |= (g == j->grain_f[(xp * n1 + y) * n2 + z]) << 0;
                m |= (g == j->grain_f[(xm * n1 + y) * n2 + z]) << 1;
                m |= (g == j->grain_f[(x * n1 + yp) * n2 + z]) << 2;
                m |= (g == j->grain_f[(x * n1 + ym) * n2 + z]) << 3;
                m |= (g == j->grain_f[(x * n1 + y) * n2 + zp]) << 4;
                m |= (g == j->grain_f[(x * n1 + ym) * n2 + z]) << 5;
                j->gb[v] = m;
            }
}

void evo_set_gnd(evo_job *j, int on) { j->gnd = on ? 1 : 0; }

evo_job *evo_open(const char *input_path, const char *rho0_path, char *err, int errlen)
{
    evo_job *j = calloc(1, sizeof(evo_job));
    char path[1024];
    int i, a, b, v, ph;
    double dev6[6], D6[6];
    t2 dev;
    if (!j) return 0;
    if (read_namelist(input_path, &j->nl)) {
        set_err(err, errlen, "cannot read namelist ", input_path);
        free(j);
        return 0;
    }
    j->n0 = j->nl.CellDim[0]; j->n1 = j->nl.CellDim[1]; j->n2 = j->nl.CellDim[2];
    j->N = j->n0 * j->n1 * j->n2;
    if (j->N <= 0 || j->nl.N_phases < 1 || j->nl.N_phases > NPH) {
        set_err(err, errlen, "bad CellDim/N_phases", 0);
        free(j);
        return 0;
    }
    j->WGT = 1. / j->N;
    if (alloc_fields(j)) { set_err(err, errlen, "out of memory", 0); evo_close(j); return 0; }
    make_B(j->B);
    /* init.c:816-854 (DD_CU off: constants from the namelist) */
    if (!j->nl.Type_phases[0]) {
        j->Shear_G[0] = shear_modulus(j->nl.ElastConst_PhaseI);
        cubic_C(j->nl.ElastConst_PhaseI, j->Cijkl[0]);
        resolve(input_path, j->nl.Slip_PhaseI, path, sizeof path);
        if (plastic_init(j, path, 0)) {
            set_err(err, errlen, "cannot read slip file ", path); evo_close(j); return 0;
        }
    }
    if (j->nl.N_phases == 2 && !j->nl.Type_phases[1]) {
        j->Shear_G[1] = shear_modulus(j->nl.ElastConst_PhaseII);
        cubic_C(j->nl.ElastConst_PhaseII, j->Cijkl[1]);
        resolve(input_path, j->nl.Slip_PhaseII, path, sizeof path);
        if (plastic_init(j, path, 1)) {
            set_err(err, errlen, "cannot read slip file ", path); evo_close(j); return 0;
        }
    }
    resolve(input_path, j->nl.initial_ms, path, sizeof path);
    if (init_microstructure(j, path)) {
        set_err(err, errlen, "cannot read microstructure ", path); evo_close(j); return 0;
    }
    /* boundary conditions, init.c:865-901 */
    for (i = 0; i < 6; i++) j->nl.VelGrad_BC[i] *= j->nl.VelGrad_BC_Flag[i];
    voigt_to_full(j->nl.VelGrad_BC, j->Udot);
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            j->Udot_s[a][b] = (j->Udot[a][b] + j->Udot[b][a]) / 2.;
            j->Udot_a[a][b] = (j->Udot[a][b] - j->Udot[b][a]) / 2.;
        }
    t2_to_v(j->B, j->Udot_s, D6, 6);
    for (i = 0; i < 5; i++) dev6[i] = D6[i];
    v_to_t2(j->B, dev6, dev, 5);
    j->d_vm = 0.0;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) j->d_vm += pow(dev[a][b], 2.0);
    j->d_vm = sqrt(2. / 3. * j->d_vm);
    for (i = 0; i < 6; i++)
        if ((j->nl.Stress_BC_Flag[i] * j->nl.VelGrad_BC_Flag[i] != 0) ||
            ((j->nl.Stress_BC_Flag[i] + j->nl.VelGrad_BC_Flag[i]) != 1)) {
            set_err(err, errlen, "inconsistent boundary conditions", 0);
            evo_close(j);
            return 0;
        }
    j->CREEP_FLAG = 0;
    for (i = 0; i < 6; i++) j->CREEP_FLAG += j->nl.Stress_BC_Flag[i];
    j->CREEP_FLAG /= 6;
    voigt_to_full(j->nl.Stress_BC, j->Scauchy);
    /* dislocation state, init.c:1068-1098 */
    for (v = 0; v < j->N; v++)
        for (i = 0; i < NS; i++) {
            j->rho_s[v][i] = j->nl.rho_SSD_initial;
            j->rho_m[v][i] = 0.0;
        }
    if (rho0_path) {
        FILE *f = fopen(rho0_path, "rb");
        if (!f) { set_err(err, errlen, "cannot open ", rho0_path); evo_close(j); return 0; }
        for (v = 0; v < j->N; v++) {
            double r;
            if (fread(&r, sizeof r, 1, f) != 1) {
                fclose(f); set_err(err, errlen, "short rho0 file", 0); evo_close(j); return 0;
            }
            for (i = 0; i < NS; i++) j->rho_s[v][i] = r;
        }
        fclose(f);
    }
    /* interaction matrices, init.c:1100-1116 */
    for (ph = 0; ph < NPH; ph++) {
        interaction(j->nl.Selfinter0[ph], j->nl.Coplanar0[ph], 0.0, 0.0, 0.0, 0.0, j->Chi[ph]);
        interaction(0.0, 0.0, j->nl.CrossSlip0[ph], j->nl.GlissileJunction0[ph],
                    j->nl.HirthLock0[ph], j->nl.LomerCottrellLock0[ph], j->Chi_1[ph]);
    }
    /* projection angles of the GND densities, init.c:1119-1140 */
    for (ph = 0; ph < NPH; ph++)
        for (i = 0; i < j->nSYS[ph]; i++)
            for (a = 0; a < j->nSYS[ph]; a++) {
                const double *ni = j->bn[ph][i], *nj = j->bn[ph][a], *bj = j->bb[ph][a];
                double sv[3], cs, c1;
                sv[0] = nj[1] * bj[2] - nj[2] * bj[1];
                sv[1] = nj[2] * bj[0] - nj[0] * bj[2];
                sv[2] = nj[0] * bj[1] - nj[1] * bj[0];
                cs = fabs(ni[0] * sv[0] + ni[1] * sv[1] + ni[2] * sv[2]);
                c1 = fabs(ni[0] * bj[0] + ni[1] * bj[1] + ni[2] * bj[2]);
                j->cos_g1[ph][i][a] = c1;
                j->sin_g1[ph][i][a] = fabs(sqrt(fabs(1.0 - c1 * c1)));
                j->cos_g2[ph][i][a] = cs;
                j->sin_g2[ph][i][a] = fabs(sqrt(fabs(1.0 - cs * cs)));
            }
    gb_masks(j);
    /* InitFields, init.c:444-516 */
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) j->DisGradAvg[a][b] = j->Udot[a][b] * j->nl.TimeStep;
    for (v = 0; v < j->N; v++) {
        const int jph = j->phase_f[v];
        if (!j->nl.Type_phases[jph - 1]) {
            t4 cg;
            int p, q;
            c66_to_t4(j->B, j->Cg[j->oid[v]], cg);
            for (a = 0; a < 3; a++)
                for (b = 0; b < 3; b++) {
                    j->Sig[v][a][b] = 0.0;
                    for (p = 0; p < 3; p++)
                        for (q = 0; q < 3; q++) j->Sig[v][a][b] += cg[a][b][p][q] * j->DisGradAvg[p][q];
                    if (j->CREEP_FLAG == 1) j->Sig[v][a][b] += j->Scauchy[a][b];
                }
        }
    }
    j->e_vm = j->d_vm * j->nl.TimeStep;
    return j;
}

void evo_close(evo_job *j)
{
    if (!j) return;
    free(j->grain_f); free(j->phase_f); free(j->oid); free(j->Cg); free(j->Sg);
    free(j->orient_key); free(j->Sig); free(j->DisGrad); free(j->Eps); free(j->Edot);
    free(j->VelGrad); free(j->TranMat); free(j->fluct); free(j->disp); free(j->Schm_gr); free(j->rho_s);
    free(j->rho_m); free(j->rho_F); free(j->rho_P); free(j->gamdot); free(j->gam_acum);
    free(j->trial_gam_acum); free(j->rho_dipole); free(j->rho_forest); free(j->rho_inplane);
    free(j->rho_dot_s); free(j->rho_tot); free(j->rho_g1); free(j->rho_g2); free(j->gb); free(j->kr); free(j->ki); free(j->fft);
    free(j->vox_e); free(j->vox_s); free(j->vox_flag);
    free(j);
}

double *evo_field(evo_job *j, const char *n)
{
    if (!strcmp(n, "Sig")) return &j->Sig[0][0][0];
    if (!strcmp(n, "DisGrad")) return &j->DisGrad[0][0][0];
    if (!strcmp(n, "Eps")) return &j->Eps[0][0][0];
    if (!strcmp(n, "Edot")) return &j->Edot[0][0][0];
    if (!strcmp(n, "VelGrad")) return &j->VelGrad[0][0][0];
    if (!strcmp(n, "TranMat")) return &j->TranMat[0][0][0];
    if (!strcmp(n, "rho_s")) return &j->rho_s[0][0];
    if (!strcmp(n, "rho_m")) return &j->rho_m[0][0];
    if (!strcmp(n, "rho_F")) return &j->rho_F[0][0];
    if (!strcmp(n, "rho_P")) return &j->rho_P[0][0];
    if (!strcmp(n, "gamdot")) return &j->gamdot[0][0];
    if (!strcmp(n, "gam_acum")) return &j->gam_acum[0][0];
    if (!strcmp(n, "trial_gam_acum")) return &j->trial_gam_acum[0][0];
    if (!strcmp(n, "rho_dipole")) return &j->rho_dipole[0][0];
    if (!strcmp(n, "rho_forest")) return &j->rho_forest[0][0];
    if (!strcmp(n, "rho_inplane")) return &j->rho_inplane[0][0];
    if (!strcmp(n, "rho_tot")) return j->rho_tot;
    if (!strcmp(n, "rho_g1")) return &j->rho_g1[0][0];
    if (!strcmp(n, "rho_g2")) return &j->rho_g2[0][0];
    if (!strcmp(n, "Schm_gr")) return &j->Schm_gr[0][0][0];
    if (!strcmp(n, "C066")) return &j->C066[0][0];
    if (!strcmp(n, "S066")) return &j->S066[0][0];
    if (!strcmp(n, "S0")) return &j->S0[0][0][0][0];
    if (!strcmp(n, "Chi")) return &j->Chi[0][0][0];
    if (!strcmp(n, "Chi_1")) return &j->Chi_1[0][0][0];
    if (!strcmp(n, "Shear_G")) return j->Shear_G;
    if (!strcmp(n, "bb_B")) return &j->bb_B[0][0];
    if (!strcmp(n, "Schm_xt")) return &j->Schm_xt[0][0][0];
    if (!strcmp(n, "scalars")) {
        /* 0..8 SigAvg, 9..17 SigAvg1, 18..26 dDisGradAvg_acum, 27 e_vm, 28 d_vm,
         * 29 s_vm, 30 s_vm1, 31 TimeTot */
        memcpy(j->scalars, j->SigAvg, 72);
        memcpy(j->scalars + 9, j->SigAvg1, 72);
        memcpy(j->scalars + 18, j->dDisGradAvg_acum, 72);
        j->scalars[27] = j->e_vm; j->scalars[28] = j->d_vm; j->scalars[29] = j->s_vm;
        j->scalars[30] = j->s_vm1; j->scalars[31] = j->TimeTot;
        return j->scalars;
    }
    return 0;
}

/* -------------------------------------------------------- hot-path parts */

/* update_schmid, kinematics.c:430-463 */
void evo_update_schmid(evo_job *j)
{
    int v;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (v = 0; v < j->N; v++) {
        const int jph = j->phase_f[v];
        int i, k, a, b, p, q;
        if (j->nl.Type_phases[jph - 1]) continue;
        for (i = 0; i < j->nSYS[jph - 1]; i++) {
            double a5[6];
            t2 aux, auxr;
            for (k = 0; k < 5; k++) a5[k] = j->Schm_xt[jph - 1][i][k];
            v_to_t2(j->B, a5, aux, 5);
            for (a = 0; a < 3; a++)
                for (b = 0; b < 3; b++) {
                    auxr[a][b] = 0.0;
                    for (p = 0; p < 3; p++)
                        for (q = 0; q < 3; q++)
                            auxr[a][b] += j->TranMat[v][a][p] * j->TranMat[v][b][q] * aux[p][q];
                }
            t2_to_v(j->B, auxr, a5, 5);
            for (k = 0; k < 5; k++) j->Schm_gr[v][i][k] = a5[k];
        }
    }
}

/* kT (evp.h:93) and the reduced activation energy (constitutive.c:543) */
static double kT_of(const evo_job *j) { return (j->nl.T__K * BOLZ * (1.0 / EV_IN_J)); }

/* StrainRate_Orowan, constitutive.c:507-728 (FORWARD_PLUS_BACKWARD; rho_F ==
 * rho_f). The GND densities enter rho_F and rho_P through their projections
 * (constitutive.c:558-577); with DD_GND off they are zero. Returns 1 on NaN. */
static int strain_rate(evo_job *j, const double *stress, double *edot, double d_edot[6][6],
                       int idx, int jph)
{
    const int p = jph - 1, ns = j->nSYS[p];
    const double kT = kT_of(j);
    const double tau_0 = j->tau0[p], shear_G = j->Shear_G[p], c_1 = j->nl.C_1[p],
                 c_2 = j->nl.C_2[p], c_3 = j->nl.C_3[p];
    const double q_slip = j->nl.Q_slip[p] * MY_J_IN_EV / kT;
    const double t_last = -1E3 * j->nl.tau_DRX * j->nl.TimeStep; /* init.c:1028 */
    double rhoS[NS], rho_f[NS], gam[NS], gam2[NS], rss[NS], tau_pass, tau_cut, tau_eff = 0,
        gam_o, tmp_gam;
    double(*sc)[5] = j->Schm_gr[idx];
    int i, k, m, bad = 0;
    for (i = 0; i < ns; i++) rhoS[i] = j->rho_s[idx][i]; /* trial_rho_s == rho_s */
    if (j->gnd) {
        /* trial_rho_g == rho_g; rho_g3 == 0 (first order) */
        const double *g1 = j->rho_g1[idx], *g2 = j->rho_g2[idx];
        for (i = 0; i < ns; i++) {
            double F = 0.0, P = 0.0;
            for (k = 0; k < ns; k++) {
                F += j->Chi_1[p][i][k] * (rhoS[k] + fabs(g1[k] * j->cos_g1[p][i][k]) +
                                          fabs(g2[k] * j->cos_g2[p][i][k]) + 0.0);
                P += j->Chi[p][i][k] * (rhoS[k] + fabs(g1[k] * j->sin_g1[p][i][k]) +
                                        fabs(g2[k] * j->sin_g2[p][i][k]) + 0.0);
            }
            j->rho_F[idx][i] = F;
            j->rho_P[idx][i] = P;
            rho_f[i] = F;
        }
    } else {
        for (i = 0; i < ns; i++) {
            double F = 0.0, P = 0.0, f = 0.0;
            for (k = 0; k < ns; k++) {
                F += j->Chi_1[p][i][k] * (rhoS[k] + 0.0 + 0.0 + 0.0);
                f += j->Chi_1[p][i][k] * (rhoS[k] + 0.0 + 0.0 + 0.0);
                P += j->Chi[p][i][k] * (rhoS[k] + 0.0 + 0.0 + 0.0);
            }
            j->rho_F[idx][i] = F;
            j->rho_P[idx][i] = P;
            rho_f[i] = f;
        }
    }
    for (i = 0; i < ns; i++) {
        tau_pass = c_1 * shear_G * j->bb_B[p][i] * sqrt(fabs(j->rho_P[idx][i] + j->rho_m[idx][i])) *
                   1.0E-3;
        tau_pass += j->nl.DeltaTau_DRX * exp((t_last - j->TimeTot) / j->nl.TimeStep / j->nl.tau_DRX);
        rss[i] = sc[i][0] * stress[0] + sc[i][1] * stress[1] + sc[i][2] * stress[2] +
                 sc[i][3] * stress[3] + sc[i][4] * stress[4];
        if (fabs(rss[i]) > tau_pass) tau_eff = (fabs(rss[i]) - tau_pass);
        tau_cut = (kT / MY_J_IN_EV) * sqrt(rho_f[i]) / c_2 / c_3 / j->bb_B[p][i] / j->bb_B[p][i] * 0.1;
        j->rho_m[idx][i] = 2.0 * kT / c_1 / c_2 / c_3 / shear_G / (pow(j->bb_B[p][i], 3.0)) *
                           sqrt(j->rho_P[idx][i] * rho_f[i]) * 160.2177;
        gam_o = 1E-3 * (j->rho_m[idx][i]) * TRIAL_FREQ_DRX * c_2 * j->bb_B[p][i] *
                exp(-1.0 * q_slip) / sqrt(rho_f[i]);
        if (fabs(rss[i]) > tau_pass) tmp_gam = gam_o * sinh(tau_eff / (tau_0 + tau_cut));
        else tmp_gam = 0.0;
        if (isnan(tmp_gam)) bad = 1;
        gam[i] = tmp_gam * ((double)(2 * (rss[i] > 0) - 1));
        if (fabs(rss[i]) > tau_pass)
            tmp_gam = gam_o * cosh(tau_eff / (tau_0 + tau_cut)) / (tau_0 + tau_cut);
        else tmp_gam = 0.0;
        if (isnan(tmp_gam)) bad = 1;
        gam2[i] = tmp_gam * (fabs(rss[i]) > tau_pass);
        j->gamdot[idx][i] = gam[i];
        j->trial_gam_acum[idx][i] = j->gam_acum[idx][i] + gam[i] * j->nl.TimeStep;
    }
    for (i = 0; i < 5; i++) {
        edot[i] = 0.;
        for (k = 0; k < ns; k++) edot[i] += sc[k][i] * gam[k];
        if (isnan(edot[i])) bad = 1;
    }
    edot[5] = 0.0;
    for (i = 0; i < 5; i++)
        for (m = 0; m < 5; m++) {
            d_edot[i][m] = 0.0;
            for (k = 0; k < ns; k++) d_edot[i][m] += sc[k][i] * sc[k][m] * gam2[k];
        }
    for (i = 0; i < 6; i++) {
        d_edot[i][5] = 0.0;
        d_edot[5][i] = 0.0;
    }
    return bad;
}

/* NR_quality, evolution.c:115-154: one flow-rule call at `sig` (with its
 * side effects on rho_m, gamdot, trial_gam_acum, rho_F, rho_P) and the
 * residual merit f = |R|^2 / 2. */
static double nr_quality(evo_job *j, const double *sig, const double *lam, const double *eps,
                         const double *str, v66 sg, int v, int jph, int *bad)
{
    double edot[6], tot[6], res[6], f;
    v66 ded;
    int a, b;
    *bad |= strain_rate(j, sig, edot, ded, v, jph);
    for (a = 0; a < 6; a++) {
        tot[a] = eps[a] + edot[a] * j->nl.TimeStep;
        for (b = 0; b < 6; b++) tot[a] += sg[a][b] * sig[b];
    }
    for (a = 0; a < 6; a++) {
        res[a] = sig[a] - lam[a];
        for (b = 0; b < 6; b++) res[a] += j->C066[a][b] * (tot[b] - str[b]);
    }
    for (f = 0.0, a = 0; a < 6; a++) f += res[a] * res[a];
    return f / 2.0;
}

/* Backtracking line search of the NR_MODIFIED build, evolution.c:280-371
 * (Numerical Recipes lnsrch with stpmax 10, ALF 1e-4, TOLX 1e-7). As in the
 * reference, f2 of the cubic model is never updated and stays 0. Returns 3
 * when the descent test fails (the reference aborts, evolution.c:324-328),
 * 1 on NaN. */
static int line_search(evo_job *j, int v, int jph, double *sig6, const double *old,
                       const double *res, v66 jac, v66 jinv, const double *lam6,
                       const double *eps6, const double *str6, v66 sg)
{
    double f_old = 0.0, gradf[6], step[6], sum, slope, test, temp, tmplam = 0;
    double a_coef, alam, alam2 = 0, alamin, b_coef, disc, f2 = 0.0, rhs1, rhs2;
    const double stpmax = 10.0, ALF = 1.E-4, TOLX = 1.E-7;
    int a, b, bad = 0;
    for (a = 0; a < 6; a++) f_old += res[a] * res[a];
    f_old *= 0.5;
    for (a = 0; a < 6; a++) {
        gradf[a] = 0.0;
        for (b = 0; b < 6; b++) gradf[a] += res[b] * jac[b][a];
    }
    for (a = 0; a < 6; a++) {
        step[a] = 0.0;
        for (b = 0; b < 6; b++) step[a] -= jinv[a][b] * res[b];
    }
    for (sum = 0.0, a = 0; a < 6; a++) sum += step[a] * step[a];
    sum = sqrt(sum);
    if (sum > stpmax)
        for (a = 0; a < 6; a++) step[a] *= stpmax / sum;
    for (slope = 0.0, a = 0; a < 6; a++) slope += gradf[a] * step[a];
    if (slope >= 0) return 3;
    test = 0.0;
    for (a = 0; a < 6; a++) {
        temp = fabs(step[a]) / SRX_MAX(fabs(old[a]), 1.0);
        if (temp > test) test = temp;
    }
    alamin = TOLX / test;
    alam = 1.0;
    for (;;) {
        double f_new;
        for (a = 0; a < 6; a++) sig6[a] = old[a] + alam * step[a];
        f_new = nr_quality(j, sig6, lam6, eps6, str6, sg, v, jph, &bad);
        if (alam < alamin) {
            for (a = 0; a < 6; a++) sig6[a] = old[a];
            break;
        } else if (f_new <= f_old + ALF * alam * slope) {
            break;
        } else {
            if (fabs(alam - 1.0) < 1.E-4) {
                tmplam = -slope / (2.0 * (f_new - f_old - slope));
            } else {
                rhs1 = f_new - f_old - alam * slope;
                rhs2 = f2 - f_old - alam2 * slope;
                a_coef = (rhs1 / (alam * alam) - rhs2 / (alam2 * alam2)) / (alam - alam2);
                b_coef = (-alam2 * rhs1 / (alam * alam) + alam * rhs2 / (alam2 * alam2)) / (alam - alam2);
                if (fabs(a_coef) < 1E-4) tmplam = -slope / (2.0 * b_coef);
                else {
                    disc = b_coef * b_coef - 3.0 * a_coef * slope;
                    if (disc < 0.0) tmplam = 0.5 * alam;
                    else if (b_coef <= 0.0) tmplam = (-b_coef + sqrt(disc)) / (3.0 * a_coef);
                    else tmplam = -slope / (b_coef + sqrt(disc));
                }
                if (tmplam > 0.5 * alam) tmplam = 0.5 * alam;
            }
        }
        alam2 = alam;
        alam = SRX_MAX(tmplam, 0.1 * alam);
        if (bad) break;
    }
    return bad ? 1 : 0;
}

/* One voxel of UpdateStress, evolution.c:181-423 (NR_MODIFIED off). */
static int update_stress_voxel(evo_job *j, int v)
{
    const int jph = j->phase_f[v];
    const double dt = j->nl.TimeStep;
    double lam6[6], sig6[6], eps6[6], str6[6], edot6[6], tot[6], res[6], old[6];
    v66 sg, jac, ded, jj;
    t2 aux;
    double signorm = 0.0, erral, cnr, ce = 0, cs = 0;
    int a, b, k, it = 0, bad = 0;
    if (j->nl.Type_phases[jph - 1]) {
        memset(j->Sig[v], 0, sizeof(t2));
        memset(j->Edot[v], 0, sizeof(t2));
        j->vox_e[v] = 0.0;
        j->vox_s[v] = 0.0;
        return 0;
    }
    memcpy(sg, j->Sg[j->oid[v]], sizeof(v66));
    t2_to_v(j->B, j->Sig[v], lam6, 6);
    t2_to_v(j->B, j->Sig[v], sig6, 6);
    t2_to_v(j->B, j->Eps[v], eps6, 6);
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) aux[a][b] = (j->DisGrad[v][a][b] + j->DisGrad[v][b][a]) / 2.0;
    t2_to_v(j->B, aux, str6, 6);
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) signorm += j->Sig[v][a][b] * j->Sig[v][a][b];
    signorm = sqrt(signorm);
    erral = 10 * 1E-10;
    while ((it < 500) && (fabs(erral) > fabs(1E-10))) {
        it++;
        for (a = 0; a < 6; a++) old[a] = sig6[a];
        bad |= strain_rate(j, sig6, edot6, ded, v, jph);
        for (a = 0; a < 6; a++) {
            tot[a] = eps6[a] + edot6[a] * dt;
            for (b = 0; b < 6; b++) tot[a] += sg[a][b] * sig6[b];
        }
        for (a = 0; a < 6; a++) {
            res[a] = sig6[a] - lam6[a];
            for (b = 0; b < 6; b++) res[a] += j->C066[a][b] * (tot[b] - str6[b]);
        }
        for (a = 0; a < 6; a++)
            for (b = 0; b < 6; b++) {
                jac[a][b] = (double)(a == b);
                for (k = 0; k < 6; k++) jac[a][b] += j->C066[a][k] * (sg[k][b] + ded[k][b] * dt);
            }
        if (j->nr_mode) memcpy(jj, jac, sizeof(v66));
        if (lu_inv66(jac)) return 2;
        if (!j->nr_mode) {
            for (a = 0; a < 6; a++)
                for (b = 0; b < 6; b++) sig6[a] -= jac[a][b] * res[b];
        } else {
            const int ls = line_search(j, v, jph, sig6, old, res, jj, jac, lam6, eps6, str6, sg);
            if (ls) return ls;
        }
        cnr = 0.0; ce = 0.0; cs = 0.0;
        for (a = 0; a < 6; a++) {
            cnr += (sig6[a] - old[a]) * (sig6[a] - old[a]);
            ce += (tot[a] - str6[a]) * (tot[a] - str6[a]);
            cs += (sig6[a] - lam6[a]) * (sig6[a] - lam6[a]);
        }
        erral = sqrt(cnr) / signorm;
        cs = sqrt(cs);
        ce = sqrt(ce);
    }
    v_to_t2(j->B, sig6, j->Sig[v], 6);
    v_to_t2(j->B, edot6, j->Edot[v], 6);
    j->vox_s[v] = cs;
    j->vox_e[v] = ce;
    return bad;
}

int evo_update_stress(evo_job *j, double *err_e, double *err_s)
{
    int v, st = 0;
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 64)
    for (v = 0; v < j->N; v++) j->vox_flag[v] = update_stress_voxel(j, v);
    *err_e = 0.0;
    *err_s = 0.0;
    for (v = 0; v < j->N; v++) {
        if (j->vox_flag[v] > st) st = j->vox_flag[v];
        if (j->nl.Type_phases[j->phase_f[v] - 1]) continue;
        *err_s += j->vox_s[v];
        *err_e += j->vox_e[v];
    }
    return st;
}

/* 3-D transform with the same per-pencil arithmetic as srx_fft3d, pencils
 * spread over threads. */
static void fft3d(evo_job *j, int sign)
{
    const int n0 = j->n0, n1 = j->n1, n2 = j->n2;
    const long n12 = (long)n1 * n2;
    double *d = j->fft;
    int c;
    const int nch = g_threads * 4;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (c = 0; c < nch; c++) {
        const long tot = (long)n0 * n1, lo = tot * c / nch, hi = tot * (c + 1) / nch;
        if (hi > lo) srx_fft1d_many(d + 2 * lo * n2, n2, (int)(hi - lo), 1, n2, sign);
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (c = 0; c < n0; c++) srx_fft1d_many(d + 2 * (size_t)c * (size_t)n12, n1, n2, n2, 1, sign);
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (c = 0; c < nch; c++) {
        const long lo = n12 * c / nch, hi = n12 * (c + 1) / nch;
        if (hi > lo) srx_fft1d_many(d + 2 * lo, n0, (int)(hi - lo), n12, 1, sign);
    }
}

/* k-space unit vector g(k), init.c:780-797 */
static void kvec(const evo_job *j, int x, int y, int z, double g[3])
{
    double t[3], g2;
    int m;
    t[0] = (double)(x) * (double)(1.0 / j->n0);
    t[1] = (double)(y) * (double)(1.0 / j->n1);
    t[2] = (double)(z) * (double)(1.0 / j->n2);
    for (m = 0; m < 3; m++) {
        t[m] -= round(t[m]);
        t[m] *= R_TWO_PI;
    }
    g2 = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    if ((x + y + z) == 0) {
        g2 = 1.0;
        t[0] = t[1] = t[2] = 0.0;
    }
    g2 = 1. / g2;
    for (m = 0; m < 3; m++) g[m] = t[m] * g2;
}

/* Forward FFT, Green contraction and inverse FFT with the displacement
 * gradient update: evolution.c:1157-1201, GAMMA from init.c:542-592. */
void evo_spectral(evo_job *j)
{
    const int N = j->N;
    int a, b, v;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            for (v = 0; v < N; v++) {
                j->fft[2 * v] = j->Sig[v][a][b];
                j->fft[2 * v + 1] = 0.0;
            }
            fft3d(j, -1);
            for (v = 0; v < N; v++) {
                j->kr[9 * (size_t)v + 3 * a + b] = j->fft[2 * v];
                j->ki[9 * (size_t)v + 3 * a + b] = j->fft[2 * v + 1];
            }
        }
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (v = 0; v < N; v++) {
        const int x = v / (j->n1 * j->n2), y = (v / j->n2) % j->n1, z = v % j->n2;
        double G[3][3][3][3], g[3], io[3][3], om[3][3], dr[3][3], di[3][3], det;
        int p, q, r, s;
        kvec(j, x, y, z, g);
        if (v == 0) {
            for (p = 0; p < 3; p++) for (q = 0; q < 3; q++)
                for (r = 0; r < 3; r++) for (s = 0; s < 3; s++)
                    G[p][q][r][s] = (j->nl.ElastBC == 0) ? -1.0 * j->S0[p][q][r][s] : 0.0;
        } else {
            for (p = 0; p < 3; p++)
                for (r = 0; r < 3; r++) {
                    io[p][r] = 0.0;
                    for (q = 0; q < 3; q++)
                        for (s = 0; s < 3; s++) io[p][r] += j->C0[p][q][r][s] * g[q] * g[s];
                }
            /* M3Inverse, init.c:518-540 */
            det = io[0][0] * (io[1][1] * io[2][2] - io[1][2] * io[2][1]) -
                  io[0][1] * (io[1][0] * io[2][2] - io[1][2] * io[2][0]) +
                  io[0][2] * (io[1][0] * io[2][1] - io[2][0] * io[1][1]);
            om[0][0] = io[1][1] * io[2][2] - io[1][2] * io[2][1];
            om[0][1] = io[0][2] * io[2][1] - io[0][1] * io[2][2];
            om[0][2] = io[0][1] * io[1][2] - io[0][2] * io[1][1];
            om[1][0] = io[1][2] * io[2][0] - io[1][0] * io[2][2];
            om[1][1] = io[0][0] * io[2][2] - io[0][2] * io[2][0];
            om[1][2] = io[0][2] * io[1][0] - io[0][0] * io[1][2];
            om[2][0] = io[1][0] * io[2][1] - io[1][1] * io[2][0];
            om[2][1] = io[0][1] * io[2][0] - io[0][0] * io[2][1];
            om[2][2] = io[0][0] * io[1][1] - io[0][1] * io[1][0];
            for (p = 0; p < 3; p++) for (q = 0; q < 3; q++) om[p][q] /= det;
            for (p = 0; p < 3; p++) for (q = 0; q < 3; q++)
                for (r = 0; r < 3; r++) for (s = 0; s < 3; s++)
                    G[p][q][r][s] = -1.0 * om[p][r] * g[q] * g[s];
        }
        for (p = 0; p < 3; p++)
            for (q = 0; q < 3; q++) {
                dr[p][q] = 0.0;
                di[p][q] = 0.0;
                for (r = 0; r < 3; r++)
                    for (s = 0; s < 3; s++) {
                        dr[p][q] += G[p][q][r][s] * j->kr[9 * (size_t)v + 3 * r + s];
                        di[p][q] += G[p][q][r][s] * j->ki[9 * (size_t)v + 3 * r + s];
                    }
            }
        for (p = 0; p < 3; p++)
            for (q = 0; q < 3; q++) {
                j->kr[9 * (size_t)v + 3 * p + q] = dr[p][q];
                j->ki[9 * (size_t)v + 3 * p + q] = di[p][q];
            }
    }
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            for (v = 0; v < N; v++) {
                j->fft[2 * v] = j->kr[9 * (size_t)v + 3 * a + b];
                j->fft[2 * v + 1] = j->ki[9 * (size_t)v + 3 * a + b];
            }
            fft3d(j, 1);
            for (v = 0; v < N; v++) {
                j->DisGrad[v][a][b] += j->dDisGradAvg[a][b] + j->fft[2 * v] / N;
                j->fluct[v][a][b] += j->fft[2 * v] / N;
            }
        }
}

/* get_smacro, evolution.c:590-664. s_vm reads SigDevAvg[3][3], one past
 * the array; with the oracle build's global layout that element is
 * SigAvg1[0][0] (the next object in .bss), which is what is used here. */
void evo_get_smacro(evo_job *j)
{
    static const int IJV[2][6] = {{0, 1, 2, 1, 0, 0}, {0, 1, 2, 2, 2, 1}};
    double sav6[6], sav5[6], oob;
    int a, b, v, i, k;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            double s = 0.0, s1 = 0.0;
            for (v = 0; v < j->N; v++) {
                s += j->Sig[v][a][b];
                if (j->phase_f[v] == 1) s1 += j->Sig[v][a][b];
            }
            j->SigAvg[a][b] = s;
            j->SigAvg1[a][b] = s1;
            j->SigAvg[a][b] *= j->WGT;
            j->SigAvg1[a][b] *= j->WGT / j->Wgt_ph1;
        }
    for (i = 0; i < 6; i++) {
        const int ii = IJV[0][i], jj = IJV[1][i];
        j->dDisGradAvg[ii][jj] = 0.0;
        if (j->nl.VelGrad_BC_Flag[i] == 0)
            for (k = 0; k < 6; k++) {
                const int kk = IJV[0][k], ll = IJV[1][k];
                j->dDisGradAvg[ii][jj] += j->S0[ii][jj][kk][ll] * j->nl.Stress_BC_Flag[k] *
                                          (j->Scauchy[kk][ll] - j->SigAvg[kk][ll]);
            }
    }
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) j->dDisGradAvg_acum[a][b] += j->dDisGradAvg[a][b];
    t2_to_v(j->B, j->SigAvg, sav6, 6);
    for (i = 0; i < 5; i++) sav5[i] = sav6[i];
    v_to_t2(j->B, sav5, j->SigDevAvg, 5);
    oob = j->SigAvg1[0][0];
    j->s_vm = 0.0;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            if (a != b) j->s_vm += j->SigDevAvg[a][b] * j->SigDevAvg[a][b];
            if (a == b) {
                const double d = j->SigDevAvg[a][b] - (j->SigDevAvg[1][1] + j->SigDevAvg[2][2] + oob) / 3.0;
                j->s_vm += d * d;
            }
        }
    j->s_vm = sqrt(3. / 2. * j->s_vm);
    t2_to_v(j->B, j->SigAvg1, sav6, 6);
    for (i = 0; i < 5; i++) sav5[i] = sav6[i];
    v_to_t2(j->B, sav5, j->SigDevAvg, 5);
    j->s_vm1 = 0.0;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) j->s_vm1 += j->SigDevAvg[a][b] * j->SigDevAvg[a][b];
    j->s_vm1 = sqrt(3. / 2. * j->s_vm1);
}

/* Orientation + update_orient, constitutive.c:142-273 */
static void reorient_voxel(evo_job *j, int v)
{
    const int jph = j->phase_f[v], p = jph - 1;
    t2 RotLoc, Lp = {{0}}, RotSlip, Rot, tran, om, om2, rot, tn;
    double w[3], wn, wt;
    int is, a, b, c;
    if (j->nl.Type_phases[p]) return;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            RotLoc[a][b] = (j->VelGrad[v][a][b] - j->VelGrad[v][b][a]) / 2.;
            tran[a][b] = j->TranMat[v][a][b];
        }
    for (is = 0; is < j->nSYS[p]; is++) {
        double bs[3], ns[3];
        for (a = 0; a < 3; a++) {
            bs[a] = 0.0;
            ns[a] = 0.0;
            for (b = 0; b < 3; b++) {
                bs[a] += tran[a][b] * j->bb[p][is][b];
                ns[a] += tran[a][b] * j->bn[p][is][b];
            }
        }
        for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) Lp[a][b] += bs[a] * ns[b] * j->gamdot[v][is];
    }
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) RotSlip[a][b] = (Lp[a][b] - Lp[b][a]) / 2.;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++)
            Rot[a][b] = (j->Udot_a[a][b] + RotLoc[a][b] - RotSlip[a][b]) * j->nl.TimeStep;
    w[0] = Rot[2][1];
    w[1] = Rot[0][2];
    w[2] = Rot[1][0];
    wn = 0.0;
    for (a = 0; a < 3; a++) wn += w[a] * w[a];
    wn = sqrt(wn);
    wt = tan(wn / 2.0);
    if (fabs(wn) < 1E-6) wn = 1.0;
    for (a = 0; a < 3; a++) w[a] *= wt / wn;
    om[0][0] = 0.; om[0][1] = -1. * w[2]; om[0][2] = w[1];
    om[1][0] = w[2]; om[1][1] = 0.; om[1][2] = -1. * w[0];
    om[2][0] = -1. * w[1]; om[2][1] = w[0]; om[2][2] = 0.;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            om2[a][b] = 0.0;
            for (c = 0; c < 3; c++) om2[a][b] += om[a][c] * om[c][b];
        }
    wt = wt * wt;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++)
            rot[a][b] = (double)(a == b) + 2. * (om[a][b] + om2[a][b]) / (1. + wt);
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            tn[a][b] = 0.0;
            for (c = 0; c < 3; c++) tn[a][b] += rot[a][c] * tran[c][b];
        }
    memcpy(j->TranMat[v], tn, sizeof(t2));
}

/* One directional derivative of Gradient_ShearRate (constitutive.c:881-1112)
 * from the same-grain bits of the plus and minus neighbours: backward, forward
 * or central difference, or zero with no same-grain neighbour. */
static double gb_diff(double c, double vp, double vm, int same_p, int same_m)
{
    if (!same_p && same_m) return c - vm;
    if (same_p && !same_m) return vp - c;
    if (same_p && same_m) return (vp - vm) / 2.0;
    return 0.0;
}

/* gadot_grad[v][i] (constitutive.c:881-1112, one rank: periodic neighbours) */
static void shear_rate_gradient(const evo_job *j, int v, int i, double gr[3])
{
    const int n0 = j->n0, n1 = j->n1, n2 = j->n2;
    const int x = v / (n1 * n2), y = (v / n2) % n1, z = v % n2;
    const int xp = (x + 1) % n0, xm = (x + n0 - 1) % n0, yp = (y + 1) % n1, ym = (y + n1 - 1) % n1,
              zp = (z + 1) % n2, zm = (z + n2 - 1) % n2;
    const unsigned m = j->gb[v];
    const double c = j->gamdot[v][i];
    gr[0] = gb_diff(c, j->gamdot[(xp * n1 + y) * n2 + z][i], j->gamdot[(xm * n1 + y) * n2 + z][i],
                    m & 1, (m >> 1) & 1);
    gr[1] = gb_diff(c, j->gamdot[(x * n1 + yp) * n2 + z][i], j->gamdot[(x * n1 + ym) * n2 + z][i],
                    (m >> 2) & 1, (m >> 3) & 1);
    gr[2] = gb_diff(c, j->gamdot[(x * n1 + y) * n2 + zp][i], j->gamdot[(x * n1 + y) * n2 + zm][i],
                    (m >> 4) & 1, (m >> 5) & 1);
}

/* DislocationEvolution, constitutive.c:1353-1529 (istep <= 2000000 branch;
 * GND part first order, constitutive.c:1428-1522). Uses rho_F, rho_m and
 * gamdot of the last flow-rule call. `grad`: the slip-rate gradients were
 * formed this increment (Hard_Flag == 1 && istep > 1, evolution.c:1348-1357);
 * otherwise gadot_grad still holds its initial zeros. */
static void dislocation_voxel(evo_job *j, int v, int grad)
{
    const int jph = j->phase_f[v], p = jph - 1;
    const double kT = kT_of(j), dt = j->nl.TimeStep, T__K = j->nl.T__K;
    const double c_4 = j->nl.C_4[p], c_5 = j->nl.C_5[p], c_6 = j->nl.C_6[p];
    const double q_bulk = j->nl.Q_bulk[p] * MY_J_IN_EV / kT, shear_G = j->Shear_G[p];
    const double nu = j->nl.ElastConst_PhaseI[3], D_0 = j->nl.D_0;
    double sig6[6], rss[NS], hydro, d_dip, dot;
    int i;
    if (j->nl.Type_phases[p]) return;
    t2_to_v(j->B, j->Sig[v], sig6, 6);
    for (i = 0; i < j->nSYS[p]; i++) {
        const double *sc = j->Schm_gr[v][i];
        rss[i] = sc[0] * sig6[0] + sc[1] * sig6[1] + sc[2] * sig6[2] + sc[3] * sig6[3] + sc[4] * sig6[4];
    }
    for (i = 0; i < j->nSYS[p]; i++) {
        const double b = j->bb_B[p][i];
        double clim;
        d_dip = sqrt(3.0) * shear_G * b / 16.0 / R_PI / (1 - nu) / (fabs(rss[i]) + EPSILON_STRESS);
        hydro = shear_G * b / R_PI / (1 - nu) / d_dip;
        clim = 1E-17 * j->rho_tot[v] * 0.5 * 1E24 * (d_dip) * (D_0 / b) * pow(j->rho_s[v][i], 2.0) *
               (exp(fabs(hydro) * b * b * b * 100 / (1.38 * T__K)) - 1.0) * exp(-1.0 * q_bulk);
        j->rho_dipole[v][i] += (clim) * dt;
        j->rho_forest[v][i] += fabs(j->gamdot[v][i]) * (c_4 * sqrt(j->rho_F[v][i])) * dt;
        j->rho_inplane[v][i] += fabs(j->gamdot[v][i]) * (c_5 * j->rho_s[v][i]) * dt;
        dot = fabs(j->gamdot[v][i]) * (c_4 * sqrt(j->rho_F[v][i]) + c_6 * (d_dip) * j->rho_m[v][i] -
                                       c_5 * j->rho_s[v][i]) -
              clim;
        j->rho_s[v][i] += dot * dt;
        j->rho_dot_s[v][i] = dot;
        j->gam_acum[v][i] = j->trial_gam_acum[v][i];
        if (j->gnd) {
            double gr[3] = {0.0, 0.0, 0.0}, gnd1, dot_g;
            const double *bp = j->bp[p][i], *bb = j->bb[p][i];
            if (grad) shear_rate_gradient(j, v, i, gr);
            gnd1 = gr[0] * bp[0] + gr[1] * bp[1] + gr[2] * bp[2];
            dot_g = gnd1 / b / j->nl.L0;
            j->rho_g1[v][i] += dot_g * dt;
            gnd1 = gr[0] * bb[0] + gr[1] * bb[1] + gr[2] * bb[2];
            dot_g = -1.0 * gnd1 / b / j->nl.L0;
            j->rho_g2[v][i] += dot_g * dt;
        }
    }
}

/* AvgDislocation, constitutive.c:1681-1808 */
static void avg_dislocation(evo_job *j)
{
    double(*arr[8])[NS] = {j->rho_F, j->rho_P, j->rho_s, j->rho_m, 0,
                           j->rho_dipole, j->rho_forest, j->rho_inplane};
    int q, v, i;
    for (q = 0; q < 8; q++) {
        double s = 0.0;
        for (v = 0; v < j->N; v++) {
            const int p = j->phase_f[v] - 1;
            if (j->nl.Type_phases[p]) continue;
            for (i = 0; i < j->nSYS[p]; i++)
                s += arr[q] ? arr[q][v][i]
                            : sqrt(j->rho_g1[v][i] * j->rho_g1[v][i] + j->rho_g2[v][i] * j->rho_g2[v][i] +
                                   0.0 * 0.0);
        }
        j->rho_avg[q] = s;
        j->rho_avg[q] *= 1.0 / j->N;
    }
}

static FILE *g_err_log = 0;

/* One pass of the equilibrium loop body (evolution.c:1151-1257) on the
 * current state; the increment head must have run (evo_begin). Used as the
 * bounded CPU sample of the hot path. */
int evo_iteration(evo_job *j)
{
    double ee, es;
    int st;
    evo_spectral(j);
    st = evo_update_stress(j, &ee, &es);
    if (st) return st;
    j->Err_e = ee * j->WGT;
    j->Err_s = es * j->WGT;
    evo_get_smacro(j);
    if (fabs(j->e_vm) < 1E-5) j->Err_e = 0.0;
    else j->Err_e /= j->e_vm;
    j->Err_s /= j->s_vm;
    return 0;
}

/* Increment head (evolution.c:1030-1141) without the loop. */
void evo_begin(evo_job *j)
{
    int v, a, b;
    for (v = 0; v < j->N; v++)
        for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) {
                j->VelGrad[v][a][b] = j->DisGrad[v][a][b];
                j->DisGrad[v][a][b] += j->Udot[a][b] * j->nl.TimeStep;
            }
    evo_update_schmid(j);
    memset(j->dDisGradAvg, 0, sizeof(t2));
    memset(j->dDisGradAvg_acum, 0, sizeof(t2));
}

int evo_increment(evo_job *j, int istep, int *iters)
{
    const double dt = j->nl.TimeStep, Err = j->nl.Err;
    const int N = j->N;
    int v, a, b, it = 0, st = 0;
    double ee, es;
    /* rho_tot from the state before the increment, evolution.c:1030-1048 */
    for (v = 0; v < N; v++) {
        const int p = j->phase_f[v] - 1;
        int i;
        j->rho_tot[v] = 0.0;
        for (i = 0; i < j->nSYS[p]; i++)
            j->rho_tot[v] += j->rho_s[v][i] + j->rho_m[v][i] +
                             sqrt(pow(j->rho_g1[v][i], 2.0) + pow(j->rho_g2[v][i], 2.0) + pow(0.0, 2.0));
    }
    /* evolution.c:1115-1128 */
    for (v = 0; v < N; v++)
        for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) {
                j->VelGrad[v][a][b] = j->DisGrad[v][a][b];
                if (j->CREEP_FLAG == 1) j->DisGrad[v][a][b] = j->DisGradAvg_actual[a][b];
                else j->DisGrad[v][a][b] += j->Udot[a][b] * dt;
            }
    /* evolution.c:1130-1132; with Update_Flag 0 the reference leaves Schm_gr
     * unset on istep 0 (undefined), rotated here instead. */
    if (istep <= 1 || j->nl.Update_Flag == 1) evo_update_schmid(j);
    memset(j->dDisGradAvg, 0, sizeof(t2));
    memset(j->dDisGradAvg_acum, 0, sizeof(t2));
    j->Err_e = 2. * Err;
    j->Err_s = 2. * Err;
    /* equilibrium loop, evolution.c:1150-1260 */
    while ((it < j->nl.IterMax) && (SRX_MAX(fabs(j->Err_s), fabs(j->Err_e)) > Err)) {
        it++;
        evo_spectral(j);
        st = evo_update_stress(j, &ee, &es);
        if (st) break;
        j->Err_e = ee;
        j->Err_s = es;
        j->Err_e *= j->WGT;
        j->Err_s *= j->WGT;
        evo_get_smacro(j);
        if (fabs(j->e_vm) < 1E-5) j->Err_e = 0.0;
        else j->Err_e /= j->e_vm;
        j->Err_s /= j->s_vm;
        if (g_err_log)
            fprintf(g_err_log, "%d %d %.17g %.17g %.17g\n", istep, it, j->Err_e, j->Err_s, j->s_vm);
    }
    if (iters) *iters = it;
    if (st) return st;
    /* evolution.c:1268-1301 */
    for (v = 0; v < N; v++)
        for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) j->VelGrad[v][a][b] = (j->DisGrad[v][a][b] - j->VelGrad[v][a][b]) / dt;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            j->DisGradAvg_actual[a][b] = j->DisGradAvg[a][b] + j->dDisGradAvg_acum[a][b];
            j->VelGradAvg[a][b] = (j->DisGradAvg_actual[a][b] - j->DisGradAvg_t[a][b]) / dt;
        }
    j->e_vm = von_mises(j->DisGradAvg_actual);
    j->d_vm = von_mises(j->VelGradAvg);
    j->TimeTot += dt;
    memcpy(j->DisGradAvg_t, j->DisGradAvg_actual, sizeof(t2));
    for (v = 0; v < N; v++)
        for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) j->Eps[v][a][b] += j->Edot[v][a][b] * dt;
    /* evolution.c:1307-1332 */
    {
        t2 el = {{0}}, dl = {{0}};
        for (v = 0; v < N; v++)
            for (a = 0; a < 3; a++)
                for (b = 0; b < 3; b++) {
                    el[a][b] += j->Eps[v][a][b] * j->WGT;
                    dl[a][b] += j->Edot[v][a][b] * j->WGT;
                }
        memcpy(j->EpsAvg, el, sizeof(t2));
        memcpy(j->EdotAvg, dl, sizeof(t2));
        j->evmp = 0.0;
        j->dvmp = 0.0;
        for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) {
                j->evmp += j->EpsAvg[a][b] * j->EpsAvg[a][b];
                j->dvmp += j->EdotAvg[a][b] * j->EdotAvg[a][b];
            }
        j->evmp = sqrt(2. / 3. * j->evmp);
        j->dvmp = sqrt(2. / 3. * j->dvmp);
    }
    /* evolution.c:1340-1343, 1361-1362 */
    if ((j->nl.Update_Flag == 1) && (istep > 1)) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (v = 0; v < N; v++) reorient_voxel(j, v);
    }
    {
        const int grad = (j->nl.Hard_Flag == 1) && (istep > 1);
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (v = 0; v < N; v++) dislocation_voxel(j, v, grad);
    }
    avg_dislocation(j);
    /* evolution.c:1401-1425: displacement_fluct[mi] = -Re(IFFT(FFT(fluct[mi][2])))/N */
    for (a = 0; a < 3; a++) {
        for (v = 0; v < N; v++) {
            j->fft[2 * v] = j->fluct[v][a][2];
            j->fft[2 * v + 1] = 0.0;
        }
        fft3d(j, -1);
        fft3d(j, 1);
        for (v = 0; v < N; v++) j->disp[v][a] = -j->fft[2 * v] / N;
    }
    /* evolution.c:1513-1515 */
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) j->DisGradAvg[a][b] = j->DisGradAvg_t[a][b] + j->Udot[a][b] * dt;
    return 0;
}

/* ----------------------------------------------------------------- output */

static void write_doubles(const char *dir, const char *name, const double *x, int n)
{
    char p[1200];
    FILE *f;
    snprintf(p, sizeof p, "%s/%s", dir, name);
    f = fopen(p, "wb");
    if (!f) return;
    fwrite(x, sizeof(double), (size_t)n, f);
    fclose(f);
}

/* WriteEpsMPI/WriteElsMPI/WriteSigMPI/WriteRhoMPI/WriteTextureMPI/
 * WriteSLIPMPI/WriteDDMPI record layouts, io.c:322-995 */
static void write_iout(evo_job *j, const char *dir, int step)
{
    const int N = j->N;
    double *tmp = malloc(sizeof(double) * (size_t)N);
    char name[200], p[1200];
    int c, v, i;
    static const int ci[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};
    for (c = 0; c < 6; c++) {
        const int a = ci[c][0], b = ci[c][1];
        for (v = 0; v < N; v++) tmp[v] = j->Eps[v][a][b];
        snprintf(name, sizeof name, "eps_%01d_S%06d.iout", c + 1, step);
        write_doubles(dir, name, tmp, N);
        for (v = 0; v < N; v++)
            tmp[v] = (c < 3) ? j->DisGrad[v][a][a] - j->Eps[v][a][a]
                             : (j->DisGrad[v][a][b] + j->DisGrad[v][b][a]) / 2.0 - j->Eps[v][a][b];
        snprintf(name, sizeof name, "els_%01d_S%06d.iout", c + 1, step);
        write_doubles(dir, name, tmp, N);
        for (v = 0; v < N; v++) tmp[v] = j->Sig[v][a][b];
        snprintf(name, sizeof name, "sig_afterDRX_%01d_S%06d.iout", c + 1, step);
        write_doubles(dir, name, tmp, N);
    }
    for (v = 0; v < N; v++) {
        const int p2 = j->phase_f[v] - 1;
        tmp[v] = 0.0;
        for (i = 0; i < j->nSYS[p2]; i++) tmp[v] += j->rho_s[v][i];
    }
    snprintf(name, sizeof name, "rho_afterDRX_SSD_S%06d.iout", step);
    write_doubles(dir, name, tmp, N);
    free(tmp);
    {
        FILE *f;
        unsigned char rec[104];
        snprintf(p, sizeof p, "%s/tex_afterDRX_S%06d.iout", dir, step);
        f = fopen(p, "wb");
        for (v = 0; f && v < N; v++) {
            t2 sa;
            double ang[3];
            int co[6];
            int a, b;
            for (a = 0; a < 3; a++)
                for (b = 0; b < 3; b++) sa[a][b] = j->TranMat[v][b][a];
            a_to_euler(sa, &ang[0], &ang[1], &ang[2]);
            co[0] = v / (j->n1 * j->n2) + 1; co[1] = (v / j->n2) % j->n1 + 1; co[2] = v % j->n2 + 1;
            co[3] = j->grain_f[v]; co[4] = j->phase_f[v]; co[5] = 0;
            memcpy(rec, ang, 24);
            memcpy(rec + 24, co, 24);
            fwrite(rec, 1, 48, f);
        }
        if (f) fclose(f);
        snprintf(p, sizeof p, "%s/slip_afterDRX_S%04d.iout", dir, step);
        f = fopen(p, "wb");
        for (v = 0; f && v < N; v++) {
            memset(rec, 0, sizeof rec);
            memcpy(rec, &j->grain_f[v], 4);
            memcpy(rec + 8, j->trial_gam_acum[v], 96);
            fwrite(rec, 1, 104, f);
        }
        if (f) fclose(f);
        snprintf(p, sizeof p, "%s/dislocation_afterDRX_S%04d.iout", dir, step);
        f = fopen(p, "wb");
        for (v = 0; f && v < N; v++) {
            memset(rec, 0, sizeof rec);
            memcpy(rec, &j->grain_f[v], 4);
            memcpy(rec + 8, j->rho_s[v], 96);
            fwrite(rec, 1, 104, f);
        }
        if (f) fclose(f);
        /* WriteNewPositionMPI (io.c:723-790) with new_position from
         * evolution.c:1434-1438: new_position + displacement_fluct - x */
        snprintf(p, sizeof p, "%s/new_position_afterDRX_S%04d.iout", dir, step);
        f = fopen(p, "wb");
        for (v = 0; f && v < N; v++) {
            const double px = (double)(v / (j->n1 * j->n2)), py = (double)((v / j->n2) % j->n1),
                         pz = (double)(v % j->n2);
            const t2 *D = &j->DisGrad[v];
            double np[3], ss[3];
            np[0] = (1.0 + (*D)[0][0]) * px + (*D)[0][1] * py + (*D)[0][2] * pz;
            np[1] = (1.0 + (*D)[1][1]) * py + (*D)[1][0] * px + (*D)[1][2] * pz;
            np[2] = (1.0 + (*D)[2][2]) * pz + (*D)[2][0] * px + (*D)[2][1] * py;
            ss[0] = np[0] + j->disp[v][0] - px;
            ss[1] = np[1] + j->disp[v][1] - py;
            ss[2] = np[2] + j->disp[v][2] - pz;
            fwrite(ss, sizeof(double), 3, f);
        }
        if (f) fclose(f);
    }
}

int evo_run(evo_job *j, const char *outdir, int nsteps, int write_iout_flag)
{
    char p[1200];
    FILE *fvm, *fdd, *ferr, *fit;
    int istep, it, st = 0;
    if (nsteps < 0) nsteps = j->nl.N_steps;
    snprintf(p, sizeof p, "%s/vm.out", outdir); fvm = fopen(p, "w");
    snprintf(p, sizeof p, "%s/dd.out", outdir); fdd = fopen(p, "w");
    snprintf(p, sizeof p, "%s/err.out", outdir); ferr = fopen(p, "w");
    snprintf(p, sizeof p, "%s/iters.txt", outdir); fit = fopen(p, "w");
    snprintf(p, sizeof p, "%s/errors.txt", outdir); g_err_log = fopen(p, "w");
    if (!fvm || !fdd || !ferr || !fit || !g_err_log) return -1;
    fprintf(fvm, "TIME\tEVM\tEVMP\tDVM\tDVMP\tSVM\tSVMSVM_1\n");
    fprintf(fdd, "TIME\tEVM\tDD_F\tDD_P\tDD_s\tDD_m\tDD_g\n");
    fprintf(ferr, "IT\tERRE\tERRS\tSVM\n");
    for (istep = 0; istep < nsteps; istep++) {
        if (nsteps != 1) fprintf(ferr, "STEP = %d\n", istep);
        if (j->CREEP_FLAG == 1 && j->e_vm > 0.3) break;
        st = evo_increment(j, istep, &it);
        fprintf(fit, "%d %d\n", istep, it);
        if (st) break;
        fprintf(fdd, "%e\t%e\t%e\t%e\t%e\t%e\t%e\n", j->TimeTot, j->e_vm, j->rho_avg[2],
                j->rho_avg[3], j->rho_avg[5], j->rho_avg[7], j->rho_avg[6]);
        fprintf(fvm, "%e\t%e\t%e\t%e\t%e\t%e\t%e\n", j->TimeTot, j->e_vm, j->evmp, j->d_vm,
                j->dvmp, j->s_vm, j->s_vm1);
        if (write_iout_flag && j->nl.PrintControl[0] == 1 && j->nl.PrintControl[1] > 0 &&
            istep % j->nl.PrintControl[1] == 0)
            write_iout(j, outdir, istep);
    }
    fclose(fvm); fclose(fdd); fclose(ferr); fclose(fit); fclose(g_err_log);
    g_err_log = 0;
    return st;
}

#ifdef SRX_ORACLE_MAIN
int main(int argc, char **argv)
{
    const char *input = 0, *outdir = ".", *rho0 = 0;
    int steps = -1, threads = 1, iout = 0, a, st, nrmode = 0, gnd = 0;
    char err[512];
    evo_job *j;
    for (a = 1; a < argc; a++) {
        if (!strcmp(argv[a], "--outdir") && a + 1 < argc) outdir = argv[++a];
        else if (!strcmp(argv[a], "--steps") && a + 1 < argc) steps = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--threads") && a + 1 < argc) threads = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--rho0") && a + 1 < argc) rho0 = argv[++a];
        else if (!strcmp(argv[a], "--iout")) iout = 1;
        else if (!strcmp(argv[a], "--line-search")) nrmode = 1;
        else if (!strcmp(argv[a], "--gnd")) gnd = 1;
        else input = argv[a];
    }
    if (!input) {
        fprintf(stderr, "usage: evp_oracle <input> [--outdir D] [--steps K] [--threads T] [--rho0 F] [--iout] [--line-search] [--gnd]\n");
        return 2;
    }
    evo_set_threads(threads);
    j = evo_open(input, rho0, err, sizeof err);
    if (!j) { fprintf(stderr, "evp_oracle: %s\n", err); return 1; }
    evo_set_nr_mode(j, nrmode);
    evo_set_gnd(j, gnd);
    st = evo_run(j, outdir, steps, iout);
    evo_close(j);
    return st;
}
#endif
