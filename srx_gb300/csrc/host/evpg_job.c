/*
 * Host driver of the GB300 EVP-FFT path: reads the reference's own input
 * files, performs SetupJob's host math and runs Evolution()'s increment loop
 * through the C ABI of include/evpg.h. Plain C99.
 *
 *   namelist        GetNameList, io.c:96-164 (key table io.c:25-94)
 *   slip systems    PlasticInit, init.c:52-231
 *   microstructure  InitMicroStruct, init.c:233-396
 *   set-up          SetupJob, init.c:728-1216; InitFields init.c:444-516
 *   increment loop  Evolution, evolution.c:667-1551 (macro bookkeeping on the
 *                   host in FP64, per-voxel work on the device)
 *   outputs         vm.out / dd.out / err.out (io.c:213-245,
 *                   evolution.c:1364-1365,1444-1446) and the .iout dumps of
 *                   WriteEpsMPI/WriteElsMPI/WriteSigMPI/WriteRhoMPI/
 *                   WriteTextureMPI/WriteSLIPMPI/WriteDDMPI (io.c:322-995)
 *
 * The set-up arithmetic keeps the reference's order of operations so the
 * device starts from the same bits as the reference.
 */
#include "evpg.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define NPH 2
#define NS EVPG_NSYS
#define R_PI 3.14159265359
#define R_TWO_PI 6.28318530718
#define EV_IN_J 1.60217733e-19
#define MY_J_IN_EV 0.62415063631
#define BOLZ 1.380658e-23

typedef double t2[3][3];
typedef double v66[6][6];
typedef double t4[3][3][3][3];

typedef struct {
    int CellDim[3], N_phases, Type_phases[2], N_steps, Update_Flag, Hard_Flag, Tex_Flag;
    int IterMax, PrintControl[2], VelGrad_BC_Flag[6], Stress_BC_Flag[6], ElastBC;
    double TimeStep, Err, VelGrad_BC[6], Stress_BC[6], ElastConst_PhaseI[4],
        ElastConst_PhaseII[4];
    char Slip_PhaseI[100], Slip_PhaseII[100], initial_ms[100];
    double a0[2], L0, T__K, Q_slip[2], Q_bulk[2], C_1[2], C_2[2], C_3[2], C_4[2], C_5[2], C_6[2],
        Selfinter0[2], Coplanar0[2], CrossSlip0[2], GlissileJunction0[2], HirthLock0[2],
        LomerCottrellLock0[2], rho_SSD_initial, D_0, tau_DRX, DeltaTau_DRX;
} evpg_namelist;

typedef struct evpg_job {
    evpg_namelist nl;
    int n0, n1, n2, N;
    void *ctx;
    double B[6][3][3];
    int nSYS[NPH];
    double tau0[NPH], Shear_G[NPH];
    double bn[NPH][NS][3], bb[NPH][NS][3], bb_B[NPH][NS], Schm_xt[NPH][NS][5];
    t4 Cijkl[NPH];
    double Chi[NPH][NS][NS], Chi_1[NPH][NS][NS];
    int *grain_f, *phase_f, *oid;
    int n_orient;
    double *okey;
    v66 *Cg, *Sg;
    v66 C066, S066;
    t4 C0, S0;
    double Wgt_ph1, WGT;
    t2 Udot, Udot_s, Udot_a, Scauchy;
    int CREEP_FLAG;
    double d_vm, e_vm, s_vm, s_vm1, evmp, dvmp, TimeTot;
    t2 DisGradAvg, DisGradAvg_t, DisGradAvg_actual, VelGradAvg, SigAvg, SigAvg1, EpsAvg, EdotAvg;
    double rho_avg[8];
    long long nr_iters;
    FILE *err_log;
    int precision, nr_mode, gnd;
    t2 dE_unapplied;  /* sum over increments of the last iteration's dDisGradAvg */
} evpg_job;

/* ------------------------------------------------------------- parsing */

enum { NI, NR, NSTR };
typedef struct { const char *name; void *ptr; int type, len, status; } nlent;

/* GetNameList, io.c:96-164 */
/* Reentrant tokenizer with strtok_r semantics (loader threads of the server
 * parse namelists concurrently; strtok keeps process-wide state). */
static char *tok_next(char *str, const char *delim, char **save)
{
    char *s = str ? str : *save, *e;
    if (!s) return NULL;
    s += strspn(s, delim);
    if (!*s) {
        *save = s;
        return NULL;
    }
    e = s + strcspn(s, delim);
    if (*e) {
        *e = 0;
        *save = e + 1;
    } else {
        *save = e;
    }
    return s;
}

static int read_namelist(const char *path, evpg_namelist *nl)
{
    nlent t[] = {
        {"CellDim", nl->CellDim, NI, 3, 0}, {"N_phases", &nl->N_phases, NI, 1, 0},
        {"Type_phases", nl->Type_phases, NI, 2, 0}, {"TimeStep", &nl->TimeStep, NR, 1, 0},
        {"N_steps", &nl->N_steps, NI, 1, 0}, {"Update_Flag", &nl->Update_Flag, NI, 1, 0},
        {"Hard_Flag", &nl->Hard_Flag, NI, 1, 0}, {"Tex_Flag", &nl->Tex_Flag, NI, 1, 0},
        {"IterMax", &nl->IterMax, NI, 1, 0}, {"PrintControl", nl->PrintControl, NI, 2, 0},
        {"Err", &nl->Err, NR, 1, 0}, {"VelGrad_BC_Flag", nl->VelGrad_BC_Flag, NI, 6, 0},
        {"VelGrad_BC", nl->VelGrad_BC, NR, 6, 0}, {"Stress_BC_Flag", nl->Stress_BC_Flag, NI, 6, 0},
        {"Stress_BC", nl->Stress_BC, NR, 6, 0}, {"ElastBC", &nl->ElastBC, NI, 1, 0},
        {"ElastConst_PhaseI", nl->ElastConst_PhaseI, NR, 4, 0},
        {"ElastConst_PhaseII", nl->ElastConst_PhaseII, NR, 4, 0},
        {"Slip_PhaseI", nl->Slip_PhaseI, NSTR, 1, 0}, {"Slip_PhaseII", nl->Slip_PhaseII, NSTR, 1, 0},
        {"initial_ms", nl->initial_ms, NSTR, 1, 0}, {"a0", nl->a0, NR, 2, 0},
        {"L0", &nl->L0, NR, 1, 0},
        {"T__K", &nl->T__K, NR, 1, 0}, {"Q_slip", nl->Q_slip, NR, 2, 0},
        {"Q_bulk", nl->Q_bulk, NR, 2, 0}, {"C_1", nl->C_1, NR, 2, 0}, {"C_2", nl->C_2, NR, 2, 0},
        {"C_3", nl->C_3, NR, 2, 0}, {"C_4", nl->C_4, NR, 2, 0}, {"C_5", nl->C_5, NR, 2, 0},
        {"C_6", nl->C_6, NR, 2, 0}, {"Selfinter0", nl->Selfinter0, NR, 2, 0},
        {"Coplanar0", nl->Coplanar0, NR, 2, 0}, {"CrossSlip0", nl->CrossSlip0, NR, 2, 0},
        {"GlissileJunction0", nl->GlissileJunction0, NR, 2, 0},
        {"HirthLock0", nl->HirthLock0, NR, 2, 0},
        {"LomerCottrellLock0", nl->LomerCottrellLock0, NR, 2, 0},
        {"rho_SSD_initial", &nl->rho_SSD_initial, NR, 1, 0}, {"D_0", &nl->D_0, NR, 1, 0},
        {"tau_DRX", &nl->tau_DRX, NR, 1, 0}, {"DeltaTau_DRX", &nl->DeltaTau_DRX, NR, 1, 0},
    };
    const int nt = (int)(sizeof t / sizeof t[0]);
    char buff[200], *tok, *save = NULL;
    FILE *fp = fopen(path, "r");
    int k, j;
    if (!fp) return -1;
    memset(nl, 0, sizeof *nl);
    for (;;) {
        if (!fgets(buff, 200, fp)) break;
        if (feof(fp)) break;
        if (buff[0] == '#' || buff[0] == '\n') continue;
        tok = tok_next(buff, " \t\n", &save);
        if (!tok) break;
        for (k = 0; k < nt; k++) {
            if (strcmp(tok, t[k].name) != 0) continue;
            if (t[k].status == 0) {
                t[k].status = 1;
                for (j = 0; j < t[k].len; j++) {
                    tok = tok_next(NULL, ", \t\n", &save);
                    if (!tok) break;
                    if (t[k].type == NI) ((int *)t[k].ptr)[j] = (int)atol(tok);
                    else if (t[k].type == NR) ((double *)t[k].ptr)[j] = atof(tok);
                    else snprintf((char *)t[k].ptr, 100, "%s", tok);
                }
            }
            break;
        }
    }
    fclose(fp);
    return 0;
}

/* chg_basis opt 0, kinematics.c:28-54 */
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

static void t2_to_v(double B[6][3][3], t2 T, double *V, int n)
{
    int i, a, b;
    for (i = 0; i < n; i++) {
        V[i] = 0.0;
        for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) V[i] += T[a][b] * B[i][a][b];
    }
}

static void v_to_t2(double B[6][3][3], const double *V, t2 T, int n)
{
    int i, a, b;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            T[a][b] = 0.0;
            for (i = 0; i < n; i++) T[a][b] += V[i] * B[i][a][b];
        }
}

static void c66_to_t4(double B[6][3][3], v66 C, t4 T)
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

static void t4_to_c66(double B[6][3][3], t4 T, v66 C)
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

/* LU_inv_66, kinematics.c:282-428 (Crout LU with implicit scaling, pivot
 * floor 1e-5 -> 1e-20); 1 when a row is below 1e-5 everywhere. */
static int lu_inv66(v66 c)
{
    int indx[6], i, imax = 0, j, k, ii, ip;
    double big, dum, sum, temp, vv[6], col[6], y[6][6];
    for (i = 0; i < 6; i++) {
        big = 0.0;
        for (j = 0; j < 6; j++)
            if ((temp = fabs(c[i][j])) > big) big = temp;
        if (fabs(big) < 1E-5) return 1;
        vv[i] = 1.0 / big;
    }
    for (j = 0; j < 6; j++) {
        for (i = 0; i < j; i++) {
            sum = c[i][j];
            for (k = 0; k < i; k++) sum -= c[i][k] * c[k][j];
            c[i][j] = sum;
        }
        big = 0.0;
        for (i = j; i < 6; i++) {
            sum = c[i][j];
            for (k = 0; k < j; k++) sum -= c[i][k] * c[k][j];
            c[i][j] = sum;
            if ((dum = vv[i] * fabs(sum)) >= big) { big = dum; imax = i; }
        }
        if (j != imax) {
            for (k = 0; k < 6; k++) { dum = c[imax][k]; c[imax][k] = c[j][k]; c[j][k] = dum; }
            vv[imax] = vv[j];
        }
        indx[j] = imax;
        if (fabs(c[j][j]) < 1E-5) c[j][j] = 1.0E-20;
        if (j != 5) {
            dum = 1.0 / (c[j][j]);
            for (i = j + 1; i < 6; i++) c[i][j] *= dum;
        }
    }
    for (k = 0; k < 6; k++) {
        for (i = 0; i < 6; i++) col[i] = 0.0;
        col[k] = 1.0;
        ii = -1;
        for (i = 0; i < 6; i++) {
            ip = indx[i];
            sum = col[ip];
            col[ip] = col[i];
            if (ii >= 0) for (j = ii; j <= i - 1; j++) sum -= c[i][j] * col[j];
            else if (fabs(sum) > 1E-5) ii = i;
            col[i] = sum;
        }
        for (i = 5; i >= 0; i--) {
            sum = col[i];
            for (j = i + 1; j < 6; j++) sum -= c[i][j] * col[j];
            col[i] = sum / c[i][i];
        }
        for (i = 0; i < 6; i++) y[i][k] = col[i];
    }
    memcpy(c, y, sizeof(v66));
    return 0;
}

static double von_mises(t2 t)
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

/* InteractionStrengthMatrix, init.c:594-703 */
static void interaction(double self, double copl, double cross, double gliss, double hirth,
                        double lomer, double chi[NS][NS])
{
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

static void resolve(const char *input, const char *name, char *out, size_t n)
{
    const char *slash = strrchr(input, '/');
    if (name[0] == '/' || !slash) snprintf(out, n, "%s", name);
    else snprintf(out, n, "%.*s/%s", (int)(slash - input), input, name);
}

/* PlasticInit, init.c:52-231 */
static int plastic_init(evpg_job *j, const char *path, int phase)
{
    FILE *fp = fopen(path, "r");
    char buf[80] = {0};
    int i, k, mx, nmodes_max = 0, nmodes = 0, imode[16], nsmx = 0, isw;
    double nrsx, g0, tw, t0f = 0, t0b, t1, th0, th1, hs, hl, norm, ax[3];
    if (!fp) return -1;
#define RD() (void)!fgets(buf, 80, fp)
    RD(); RD(); RD(); RD(); RD(); sscanf(buf, "%lf %lf %lf", &ax[0], &ax[1], &ax[2]);
    RD(); RD(); RD(); sscanf(buf, "%d", &nmodes_max);
    RD(); RD(); RD(); sscanf(buf, "%d", &nmodes);
    if (nmodes < 1 || nmodes > 16) { fclose(fp); return -2; }
    RD(); RD();
    for (i = 0; i < nmodes; i++) { RD(); sscanf(buf, "%d", &imode[i]); }
    RD();
    for (i = 0; i < nmodes_max; i++) {
        int match = 0;
        RD(); sscanf(buf, "%*s %*s %d %*s", &mx);
        for (k = 0; k < nmodes; k++) if (mx == imode[k]) { match = 1; break; }
        RD(); RD(); sscanf(buf, "%d %lf %lf %lf %d", &nsmx, &nrsx, &g0, &tw, &isw);
        RD(); RD(); sscanf(buf, "%lf %lf %lf %lf %lf", &t0f, &t0b, &t1, &th0, &th1);
        RD(); RD(); sscanf(buf, "%lf %lf", &hs, &hl);
        RD();
        if (match) {
            if (nsmx < 1 || nsmx > NS) { fclose(fp); return -3; }
            j->nSYS[phase] = nsmx;
            j->tau0[phase] = t0f;
            for (k = 0; k < nsmx; k++) {
                RD();
                sscanf(buf, "%lf %lf %lf %lf %lf %lf", &j->bn[phase][k][0], &j->bn[phase][k][1],
                       &j->bn[phase][k][2], &j->bb[phase][k][0], &j->bb[phase][k][1], &j->bb[phase][k][2]);
            }
        } else {
            for (k = 0; k < nsmx; k++) RD();
        }
    }
#undef RD
    fclose(fp);
    for (i = 0; i < nmodes; i++)
        for (k = 0; k < j->nSYS[phase]; k++) {
            t2 aux;
            double a5[6];
            int a, b;
            norm = sqrt(pow(j->bn[phase][k][0], 2.0) + pow(j->bn[phase][k][1], 2.0) + pow(j->bn[phase][k][2], 2.0));
            for (mx = 0; mx < 3; mx++) j->bn[phase][k][mx] /= norm;
            norm = sqrt(pow(j->bb[phase][k][0], 2.0) + pow(j->bb[phase][k][1], 2.0) + pow(j->bb[phase][k][2], 2.0));
            j->bb_B[phase][k] = j->nl.a0[phase] / sqrt(2.0);
            for (mx = 0; mx < 3; mx++) j->bb[phase][k][mx] /= norm;
            norm = 0.0;
            for (mx = 0; mx < 3; mx++) norm += j->bn[phase][k][mx] * j->bb[phase][k][mx];
            if (norm > 1E-3) return -4;
            for (a = 0; a < 3; a++)
                for (b = 0; b < 3; b++)
                    aux[a][b] = (j->bn[phase][k][a] * j->bb[phase][k][b] + j->bn[phase][k][b] * j->bb[phase][k][a]) / 2.0;
            t2_to_v(j->B, aux, a5, 5);
            for (mx = 0; mx < 5; mx++) j->Schm_xt[phase][k][mx] = a5[mx];
        }
    return 0;
}

/* EulerToTransMatrix opt 2 (kinematics.c:218-234) */
static void euler_to_a(double t1, double ph, double t2v, t2 a)
{
    double ct1 = cos(t1), st1 = sin(t1), cph = cos(ph), sph = sin(ph), ct2 = cos(t2v), st2 = sin(t2v);
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

/* EulerToTransMatrix opt 1 (kinematics.c:198-217), degrees */
static void a_to_euler(t2 a, double *t1, double *ph, double *t2v)
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

/* InitMicroStruct, init.c:233-396; per distinct (angles, phase) the rotated
 * stiffness and its LU inverse. Fills TranMat into tran[N][9]. */
static int init_ms(evpg_job *j, const char *path, double *tran)
{
    FILE *fp = fopen(path, "r");
    char buf[80] = {0};
    int v, cap = 64, nph1 = 0, a, b;
    v66 acc;
    if (!fp) return -1;
    memset(acc, 0, sizeof acc);
    j->okey = (double *)malloc(sizeof(double) * 4 * (size_t)cap);
    j->Cg = (v66 *)malloc(sizeof(v66) * (size_t)cap);
    j->Sg = (v66 *)malloc(sizeof(v66) * (size_t)cap);
    for (v = 0; v < j->N; v++) {
        double ph = 0, th = 0, om = 0;
        int ii = 0, jj = 0, kk = 0, jgr = 0, jph = 0, o;
        if (!fgets(buf, 80, fp)) { fclose(fp); return -2; }
        sscanf(buf, "%lf %lf %lf %d %d %d %d %d", &ph, &th, &om, &ii, &jj, &kk, &jgr, &jph);
        if (((ii - 1) * j->n1 + jj - 1) * j->n2 + kk - 1 != v || jph < 1 || jph > NPH) { fclose(fp); return -3; }
        if (jph == 1) nph1++;
        j->grain_f[v] = jgr;
        j->phase_f[v] = jph;
        j->oid[v] = -1;
        for (a = 0; a < 9; a++) tran[9 * (size_t)v + a] = 0.0;
        if (j->nl.Type_phases[jph - 1]) continue;
        {
            t2 sa;
            ph *= R_PI / 180.; th *= R_PI / 180.; om *= R_PI / 180.;
            euler_to_a(ph, th, om, sa);
            for (a = 0; a < 3; a++)
                for (b = 0; b < 3; b++) tran[9 * (size_t)v + 3 * a + b] = sa[b][a];
            for (o = 0; o < j->n_orient; o++) {
                const double *k4 = j->okey + 4 * o;
                if (k4[0] == ph && k4[1] == th && k4[2] == om && k4[3] == (double)jph) break;
            }
            if (o == j->n_orient) {
                t4 cx;
                int p, q, r, s, m, n, pp, qq;
                if (j->n_orient == cap) {
                    cap *= 2;
                    j->okey = (double *)realloc(j->okey, sizeof(double) * 4 * (size_t)cap);
                    j->Cg = (v66 *)realloc(j->Cg, sizeof(v66) * (size_t)cap);
                    j->Sg = (v66 *)realloc(j->Sg, sizeof(v66) * (size_t)cap);
                }
                /* Ten4thTransform opt 2, kinematics.c:262-274 */
                for (p = 0; p < 3; p++)
                    for (q = 0; q < 3; q++)
                        for (r = 0; r < 3; r++)
                            for (s = 0; s < 3; s++) {
                                cx[p][q][r][s] = 0.0;
                                for (m = 0; m < 3; m++)
                                    for (n = 0; n < 3; n++)
                                        for (pp = 0; pp < 3; pp++)
                                            for (qq = 0; qq < 3; qq++)
                                                cx[p][q][r][s] += sa[m][p] * sa[n][q] * sa[pp][r] * sa[qq][s] *
                                                                  j->Cijkl[jph - 1][m][n][pp][qq];
                            }
                t4_to_c66(j->B, cx, j->Cg[o]);
                memcpy(j->Sg[o], j->Cg[o], sizeof(v66));
                if (lu_inv66(j->Sg[o])) { fclose(fp); return -5; }
                j->okey[4 * o] = ph; j->okey[4 * o + 1] = th; j->okey[4 * o + 2] = om;
                j->okey[4 * o + 3] = (double)jph;
                j->n_orient++;
            }
            j->oid[v] = o;
            for (a = 0; a < 6; a++)
                for (b = 0; b < 6; b++) acc[a][b] += j->Cg[o][a][b];
        }
    }
    fclose(fp);
    j->Wgt_ph1 = (1.0 * (double)nph1) / j->N;
    for (a = 0; a < 6; a++)
        for (b = 0; b < 6; b++) {
            j->C066[a][b] = acc[a][b];
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

static void cubic_C(const double *ec, t4 c)
{
    int i, jx;
    memset(c, 0, sizeof(t4));
    for (i = 0; i < 3; i++) c[i][i][i][i] = ec[0];
    for (i = 0; i < 3; i++)
        for (jx = 0; jx < 3; jx++)
            if (i != jx) {
                c[i][i][jx][jx] = ec[1];
                c[i][jx][i][jx] = ec[2];
                c[i][jx][jx][i] = ec[2];
            }
}

static double shear_modulus(const double *ec)
{
    return 0.1 * (ec[0] - ec[1] + 3 * ec[2]) +
           (0.5) * (5 * (ec[0] - ec[1]) * ec[2]) / (4 * ec[2] + 3 * (ec[0] - ec[1]));
}

int evpg_job_close(void *jp)
{
    evpg_job *j = (evpg_job *)jp;
    if (!j) return EVPG_OK;
    if (j->ctx) evpg_destroy(j->ctx);
    free(j->grain_f); free(j->phase_f); free(j->oid); free(j->okey); free(j->Cg); free(j->Sg);
    free(j);
    return EVPG_OK;
}

int evpg_job_open(const char *input, const char *rho0, int32_t precision, int32_t nr_mode, void **out)
{
    return evpg_job_open_opts(input, rho0, precision, nr_mode, 0, out);
}

int evpg_job_open_opts(const char *input, const char *rho0, int32_t precision, int32_t nr_mode,
                       int32_t options, void **out)
{
    evpg_job *j;
    char path[1024];
    int i, a, b, v, st, p;
    double *tran = 0, *sig0 = 0, *rho = 0;
    evpg_rve_desc d;
    double kT;
    if (!input || !out) return EVPG_ERR_ARG;
    *out = 0;
    j = (evpg_job *)calloc(1, sizeof(evpg_job));
    if (!j) return EVPG_ERR_NOMEM;
    if (read_namelist(input, &j->nl)) { free(j); return EVPG_ERR_IO; }
    j->n0 = j->nl.CellDim[0]; j->n1 = j->nl.CellDim[1]; j->n2 = j->nl.CellDim[2];
    j->N = j->n0 * j->n1 * j->n2;
    if (j->N <= 0 || j->nl.N_phases < 1 || j->nl.N_phases > NPH) { free(j); return EVPG_ERR_IO; }
    j->WGT = 1. / j->N;
    make_B(j->B);
    j->grain_f = (int *)calloc((size_t)j->N, sizeof(int));
    j->phase_f = (int *)calloc((size_t)j->N, sizeof(int));
    j->oid = (int *)calloc((size_t)j->N, sizeof(int));
    tran = (double *)calloc(9 * (size_t)j->N, sizeof(double));
    sig0 = (double *)calloc(9 * (size_t)j->N, sizeof(double));
    rho = (double *)calloc(12 * (size_t)j->N, sizeof(double));
    if (!j->grain_f || !j->phase_f || !j->oid || !tran || !sig0 || !rho) { st = EVPG_ERR_NOMEM; goto bad; }
    st = EVPG_ERR_IO;
    if (!j->nl.Type_phases[0]) {
        j->Shear_G[0] = shear_modulus(j->nl.ElastConst_PhaseI);
        cubic_C(j->nl.ElastConst_PhaseI, j->Cijkl[0]);
        resolve(input, j->nl.Slip_PhaseI, path, sizeof path);
        if (plastic_init(j, path, 0)) goto bad;
    }
    if (j->nl.N_phases == 2 && !j->nl.Type_phases[1]) {
        j->Shear_G[1] = shear_modulus(j->nl.ElastConst_PhaseII);
        cubic_C(j->nl.ElastConst_PhaseII, j->Cijkl[1]);
        resolve(input, j->nl.Slip_PhaseII, path, sizeof path);
        if (plastic_init(j, path, 1)) goto bad;
    }
    resolve(input, j->nl.initial_ms, path, sizeof path);
    if (init_ms(j, path, tran)) goto bad;
    /* boundary conditions, init.c:865-901 */
    for (i = 0; i < 6; i++) j->nl.VelGrad_BC[i] *= j->nl.VelGrad_BC_Flag[i];
    voigt_to_full(j->nl.VelGrad_BC, j->Udot);
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            j->Udot_s[a][b] = (j->Udot[a][b] + j->Udot[b][a]) / 2.;
            j->Udot_a[a][b] = (j->Udot[a][b] - j->Udot[b][a]) / 2.;
        }
    {
        double D6[6], d5[6];
        t2 dev;
        t2_to_v(j->B, j->Udot_s, D6, 6);
        for (i = 0; i < 5; i++) d5[i] = D6[i];
        v_to_t2(j->B, d5, dev, 5);
        j->d_vm = 0.0;
        for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) j->d_vm += pow(dev[a][b], 2.0);
        j->d_vm = sqrt(2. / 3. * j->d_vm);
    }
    for (i = 0; i < 6; i++)
        if ((j->nl.Stress_BC_Flag[i] * j->nl.VelGrad_BC_Flag[i] != 0) ||
            ((j->nl.Stress_BC_Flag[i] + j->nl.VelGrad_BC_Flag[i]) != 1)) goto bad;
    j->CREEP_FLAG = 0;
    for (i = 0; i < 6; i++) j->CREEP_FLAG += j->nl.Stress_BC_Flag[i];
    j->CREEP_FLAG /= 6;
    voigt_to_full(j->nl.Stress_BC, j->Scauchy);
    for (p = 0; p < NPH; p++) {
        interaction(j->nl.Selfinter0[p], j->nl.Coplanar0[p], 0.0, 0.0, 0.0, 0.0, j->Chi[p]);
        interaction(0.0, 0.0, j->nl.CrossSlip0[p], j->nl.GlissileJunction0[p], j->nl.HirthLock0[p],
                    j->nl.LomerCottrellLock0[p], j->Chi_1[p]);
    }
    /* initial densities, init.c:1068-1098 (+ optional per-voxel file) */
    for (v = 0; v < j->N; v++)
        for (i = 0; i < NS; i++) rho[12 * (size_t)v + i] = j->nl.rho_SSD_initial;
    if (rho0) {
        FILE *f = fopen(rho0, "rb");
        if (!f) goto bad;
        for (v = 0; v < j->N; v++) {
            double r;
            if (fread(&r, sizeof r, 1, f) != 1) { fclose(f); goto bad; }
            for (i = 0; i < NS; i++) rho[12 * (size_t)v + i] = r;
        }
        fclose(f);
    }
    /* InitFields, init.c:453-495: sig = C_gr : (Udot dt) */
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) j->DisGradAvg[a][b] = j->Udot[a][b] * j->nl.TimeStep;
    {
        double *so = (double *)calloc(9 * (size_t)(j->n_orient > 0 ? j->n_orient : 1), sizeof(double));
        int o, c, e;
        for (o = 0; o < j->n_orient; o++) {
            t4 cg;
            c66_to_t4(j->B, j->Cg[o], cg);
            for (a = 0; a < 3; a++)
                for (b = 0; b < 3; b++) {
                    double s = 0.0;
                    for (c = 0; c < 3; c++)
                        for (e = 0; e < 3; e++) s += cg[a][b][c][e] * j->DisGradAvg[c][e];
                    if (j->CREEP_FLAG == 1) s += j->Scauchy[a][b];
                    so[9 * o + 3 * a + b] = s;
                }
        }
        for (v = 0; v < j->N; v++)
            if (j->oid[v] >= 0) memcpy(sig0 + 9 * (size_t)v, so + 9 * j->oid[v], 9 * sizeof(double));
        free(so);
    }
    j->e_vm = j->d_vm * j->nl.TimeStep;

    /* device descriptor */
    memset(&d, 0, sizeof d);
    d.n[0] = j->n0; d.n[1] = j->n1; d.n[2] = j->n2;
    d.n_orient = j->n_orient;
    d.voxel_orient = j->oid;
    d.voxel_phase = j->phase_f;
    {
        double *cg = (double *)malloc(sizeof(v66) * (size_t)(j->n_orient > 0 ? j->n_orient : 1));
        double *sg = (double *)malloc(sizeof(v66) * (size_t)(j->n_orient > 0 ? j->n_orient : 1));
        if (!cg || !sg) { free(cg); free(sg); st = EVPG_ERR_NOMEM; goto bad; }
        memcpy(cg, j->Cg, sizeof(v66) * (size_t)j->n_orient);
        memcpy(sg, j->Sg, sizeof(v66) * (size_t)j->n_orient);
        d.c_gr = cg;
        d.s_gr = sg;
        d.tranmat = tran;
        d.sig0 = sig0;
        d.rho_s0 = rho;
        memcpy(d.c066, j->C066, sizeof d.c066);
        memcpy(d.s066, j->S066, sizeof d.s066);
        memcpy(d.c0, j->C0, sizeof d.c0);
        memcpy(d.s0, j->S0, sizeof d.s0);
        d.wgt_ph1 = j->Wgt_ph1;
        kT = (j->nl.T__K * BOLZ * (1.0 / EV_IN_J));
        for (p = 0; p < NPH; p++) {
            evpg_phase_desc *s = &d.phase[p];
            s->crystal = !j->nl.Type_phases[p];
            s->n_sys = (p < j->nl.N_phases) ? j->nSYS[p] : 0;
            memcpy(s->schm_xt, j->Schm_xt[p], sizeof s->schm_xt);
            memcpy(s->bn, j->bn[p], sizeof s->bn);
            memcpy(s->bb, j->bb[p], sizeof s->bb);
            memcpy(s->burgers, j->bb_B[p], sizeof s->burgers);
            memcpy(s->chi, j->Chi[p], sizeof s->chi);
            memcpy(s->chi1, j->Chi_1[p], sizeof s->chi1);
            s->shear_g = j->Shear_G[p];
            s->c1 = j->nl.C_1[p]; s->c2 = j->nl.C_2[p]; s->c3 = j->nl.C_3[p];
            s->c4 = j->nl.C_4[p]; s->c5 = j->nl.C_5[p]; s->c6 = j->nl.C_6[p];
            s->q_slip = j->nl.Q_slip[p] * MY_J_IN_EV / kT;
            s->q_bulk = j->nl.Q_bulk[p] * MY_J_IN_EV / kT;
            s->tau0 = j->tau0[p];
            if (s->crystal && s->n_sys == 0) s->crystal = 0;
        }
        d.dt = j->nl.TimeStep;
        d.kT = kT;
        d.temperature = j->nl.T__K;
        d.nu = j->nl.ElastConst_PhaseI[3];
        d.d0 = j->nl.D_0;
        d.delta_tau_drx = j->nl.DeltaTau_DRX;
        d.tau_drx = j->nl.tau_DRX;
        d.elast_bc = j->nl.ElastBC;
        for (i = 0; i < 6; i++) {
            d.velgrad_bc_flag[i] = j->nl.VelGrad_BC_Flag[i];
            d.stress_bc_flag[i] = j->nl.Stress_BC_Flag[i];
        }
        memcpy(d.scauchy, j->Scauchy, sizeof d.scauchy);
        memcpy(d.udot_a, j->Udot_a, sizeof d.udot_a);
        d.err_tol = j->nl.Err;
        d.iter_max = j->nl.IterMax;
        j->precision = precision;
        j->nr_mode = nr_mode;
        d.precision = precision;
        d.nr_mode = nr_mode;
        j->gnd = (options & EVPG_JOB_GND) != 0;
        d.gnd = j->gnd;
        d.l0 = j->nl.L0;
        d.voxel_grain = j->grain_f;
        st = evpg_create(&d, &j->ctx);
        free(cg);
        free(sg);
    }
    free(tran); free(sig0); free(rho);
    if (st) { evpg_job_close(j); return st; }
    *out = j;
    return EVPG_OK;
bad:
    free(tran); free(sig0); free(rho);
    evpg_job_close(j);
    return st;
}

void *evpg_job_ctx(void *jp) { return jp ? ((evpg_job *)jp)->ctx : 0; }

int evpg_job_nvox(void *jp, int32_t n[3])
{
    evpg_job *j = (evpg_job *)jp;
    if (!j || !n) return EVPG_ERR_ARG;
    n[0] = j->n0; n[1] = j->n1; n[2] = j->n2;
    return EVPG_OK;
}

int evpg_job_nsteps(void *jp) { return jp ? ((evpg_job *)jp)->nl.N_steps : 0; }

/* Load of a namelist's VelGrad_BC_Flag/VelGrad_BC/Stress_BC_Flag/Stress_BC
 * into the job (init.c:865-901); returns nonzero for an inconsistent set. */
static int job_load(evpg_job *j, const int32_t vflag[6], const double velgrad[6], const int32_t sflag[6],
                    const double stress[6])
{
    double vg[6];
    int i, a, b;
    for (i = 0; i < 6; i++) {
        if ((sflag[i] * vflag[i] != 0) || ((sflag[i] + vflag[i]) != 1)) return EVPG_ERR_ARG;
        j->nl.VelGrad_BC_Flag[i] = vflag[i];
        j->nl.Stress_BC_Flag[i] = sflag[i];
        vg[i] = velgrad[i] * vflag[i];
        j->nl.VelGrad_BC[i] = vg[i];
        j->nl.Stress_BC[i] = stress[i];
    }
    voigt_to_full(vg, j->Udot);
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            j->Udot_s[a][b] = (j->Udot[a][b] + j->Udot[b][a]) / 2.;
            j->Udot_a[a][b] = (j->Udot[a][b] - j->Udot[b][a]) / 2.;
        }
    j->CREEP_FLAG = 0;
    for (i = 0; i < 6; i++) j->CREEP_FLAG += j->nl.Stress_BC_Flag[i];
    j->CREEP_FLAG /= 6;
    voigt_to_full(j->nl.Stress_BC, j->Scauchy);
    return EVPG_OK;
}

/* Switch the job's loading before its next increment: the applied average
 * of that increment becomes DisGradAvg_t + Udot_new*TimeStep. */
int evpg_job_set_load(void *jp, const int32_t vflag[6], const double velgrad[6], const int32_t sflag[6],
                      const double stress[6])
{
    evpg_job *j = (evpg_job *)jp;
    int st, a, b;
    if (!j || !vflag || !velgrad || !sflag || !stress) return EVPG_ERR_ARG;
    st = job_load(j, vflag, velgrad, sflag, stress);
    if (st) return st;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) j->DisGradAvg[a][b] = j->DisGradAvg_t[a][b] + j->Udot[a][b] * j->nl.TimeStep;
    return evpg_set_load(j->ctx, j->nl.VelGrad_BC_Flag, j->nl.Stress_BC_Flag, (const double(*)[3])j->Scauchy,
                         (const double(*)[3])j->Udot_a);
}

/* Load switch to the boundary conditions of another namelist file. */
int evpg_job_set_load_from(void *jp, const char *input)
{
    evpg_namelist nl;
    if (!jp || !input) return EVPG_ERR_ARG;
    memset(&nl, 0, sizeof nl);
    if (read_namelist(input, &nl)) return EVPG_ERR_IO;
    return evpg_job_set_load(jp, nl.VelGrad_BC_Flag, nl.VelGrad_BC, nl.Stress_BC_Flag, nl.Stress_BC);
}

/* Grid of a namelist file (CellDim) without opening the job. */
int evpg_job_grid(const char *input, int32_t n[3])
{
    evpg_namelist nl;
    if (!input || !n) return EVPG_ERR_ARG;
    memset(&nl, 0, sizeof nl);
    if (read_namelist(input, &nl)) return EVPG_ERR_IO;
    n[0] = nl.CellDim[0]; n[1] = nl.CellDim[1]; n[2] = nl.CellDim[2];
    return EVPG_OK;
}

/* Controls of increment istep (evolution.c:1115-1128): Udot*TimeStep,
 * creep, the applied average, TimeTot, the strain-error normaliser e_vm and
 * the tail flags: update_orient when Update_Flag == 1 && istep > 1
 * (evolution.c:1340-1343), the GND slip-rate gradients when Hard_Flag == 1
 * && istep > 1 (evolution.c:1348-1357). */
static void job_controls(const evpg_job *j, int istep, t2 udt, int *tail)
{
    const double dt = j->nl.TimeStep;
    int a, b;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) udt[a][b] = j->Udot[a][b] * dt;
    *tail = ((j->nl.Update_Flag == 1) && (istep > 1) ? EVPG_TAIL_REORIENT : 0) |
            (j->gnd && (j->nl.Hard_Flag == 1) && (istep > 1) ? EVPG_TAIL_GND_GRADIENT : 0);
}

/* Increment bookkeeping after the tail (evolution.c:1273-1332). */
static void job_finish(evpg_job *j, const evpg_iter_out *io, const evpg_incr_out *eo)
{
    const double dt = j->nl.TimeStep;
    int a, b;
    memcpy(j->SigAvg, io->sig_avg, sizeof(t2));
    memcpy(j->SigAvg1, io->sig_avg_ph1, sizeof(t2));
    /* the correction of the loop's last get_smacro enters dDisGradAvg_acum
     * but never DisGrad (the loop ends before the next update) */
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) j->dE_unapplied[a][b] += io->ddisgrad[a][b];
    j->s_vm = io->s_vm;
    j->s_vm1 = io->s_vm1;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            j->DisGradAvg_actual[a][b] = j->DisGradAvg[a][b] + io->ddisgrad_acum[a][b];
            j->VelGradAvg[a][b] = (j->DisGradAvg_actual[a][b] - j->DisGradAvg_t[a][b]) / dt;
        }
    j->e_vm = von_mises(j->DisGradAvg_actual);
    j->d_vm = von_mises(j->VelGradAvg);
    j->TimeTot += dt;
    memcpy(j->DisGradAvg_t, j->DisGradAvg_actual, sizeof(t2));
    memcpy(j->EpsAvg, eo->eps_avg, sizeof(t2));
    memcpy(j->EdotAvg, eo->edot_avg, sizeof(t2));
    j->evmp = 0.0;
    j->dvmp = 0.0;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            j->evmp += j->EpsAvg[a][b] * j->EpsAvg[a][b];
            j->dvmp += j->EdotAvg[a][b] * j->EdotAvg[a][b];
        }
    j->evmp = sqrt(2. / 3. * j->evmp);
    j->dvmp = sqrt(2. / 3. * j->dvmp);
    memcpy(j->rho_avg, eo->rho_avg, sizeof j->rho_avg);
    j->nr_iters = eo->nr_iterations;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) j->DisGradAvg[a][b] = j->DisGradAvg_t[a][b] + j->Udot[a][b] * dt;
}

/* One increment of Evolution(), evolution.c:726-1520. */
int evpg_job_increment(void *jp, int32_t istep, int32_t *iters)
{
    evpg_job *j = (evpg_job *)jp;
    t2 udt;
    evpg_iter_out io;
    evpg_incr_out eo;
    int st, tail;
    if (!j) return EVPG_ERR_ARG;
    job_controls(j, istep, udt, &tail);
    if (j->err_log) {
        st = evpg_increment_begin(j->ctx, (const double(*)[3])udt, j->CREEP_FLAG == 1,
                                  (const double(*)[3])j->DisGradAvg_actual, j->TimeTot);
        if (st) return st;
        /* one device round trip per iteration, to log the reference's lines */
        do {
            st = evpg_equilibrium_iteration(j->ctx, j->e_vm, &io);
            if (st) return st;
            fprintf(j->err_log, "%d %d %.17g %.17g %.17g\n", istep, io.iter, io.err_e, io.err_s, io.s_vm);
        } while (!io.converged && io.iter < j->nl.IterMax);
        st = evpg_increment_end(j->ctx, tail, &eo);
        if (st) return st;
    } else {
        /* the whole increment as one graph launch */
        st = evpg_increment(j->ctx, (const double(*)[3])udt, j->CREEP_FLAG == 1,
                            (const double(*)[3])j->DisGradAvg_actual, j->TimeTot, j->e_vm, tail, &io, &eo);
        if (st) return st;
    }
    if (iters) *iters = io.iter;
    job_finish(j, &io, &eo);
    return EVPG_OK;
}

/* Stage increment istep of a job into slot `slot` of a batch. */
int evpg_job_stage(void *jp, void *batch, int32_t slot, int32_t istep)
{
    evpg_job *j = (evpg_job *)jp;
    t2 udt;
    int tail;
    if (!j || !batch) return EVPG_ERR_ARG;
    job_controls(j, istep, udt, &tail);
    return evpg_batch_stage(batch, slot, (const double(*)[3])udt, j->CREEP_FLAG == 1,
                            (const double(*)[3])j->DisGradAvg_actual, j->TimeTot, j->e_vm, tail);
}

/* After a round: if the job's increment in `slot` ended, do its bookkeeping
 * and set *ended = 1 (iters: its equilibrium iterations). A slot that
 * stopped on an error returns that error. */
int evpg_job_collect(void *jp, void *batch, int32_t slot, int32_t *ended, int32_t *iters)
{
    evpg_job *j = (evpg_job *)jp;
    evpg_iter_out io;
    evpg_incr_out eo;
    int32_t phase = 0, status = 0;
    int st;
    if (!j || !batch || !ended) return EVPG_ERR_ARG;
    *ended = 0;
    st = evpg_batch_slot(batch, slot, &phase, &status, &io, &eo);
    if (st) return st;
    if (status) return status;
    if (phase != 3) return EVPG_OK;
    *ended = 1;
    if (iters) *iters = io.iter;
    job_finish(j, &io, &eo);
    return EVPG_OK;
}

/* Run increments [0, nsteps[i]) of n jobs of one precision and NR mode in
 * one batch, rounds of at most max_ticks iterations; iters[i*stride + k]
 * receives job i's iterations of increment k (stride >= max nsteps). */
int evpg_jobs_run_batched(void *const *jobs, int32_t n, const int32_t *nsteps, int32_t max_ticks,
                          int32_t *iters, int32_t stride, int64_t *rounds_out)
{
    void *batch = 0;
    void **ctxs;
    int32_t *next;
    int i, st, prec, mode, left;
    int64_t rounds = 0;
    if (!jobs || n < 1 || !nsteps || max_ticks < 1) return EVPG_ERR_ARG;
    prec = ((evpg_job *)jobs[0])->precision;
    mode = ((evpg_job *)jobs[0])->nr_mode;
    st = evpg_batch_create(prec, mode, &batch);
    if (st) return st;
    ctxs = (void **)calloc((size_t)n, sizeof(void *));
    next = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    for (i = 0; i < n; i++) ctxs[i] = ((evpg_job *)jobs[i])->ctx;
    st = evpg_batch_set(batch, ctxs, n);
    left = 0;
    for (i = 0; i < n && !st; i++)
        if (nsteps[i] > 0) {
            st = evpg_job_stage(jobs[i], batch, i, 0);
            left++;
        }
    while (!st && left > 0) {
        int32_t ticks = 0;
        st = evpg_batch_round(batch, max_ticks, &ticks);
        rounds++;
        for (i = 0; i < n && !st; i++) {
            int32_t ended = 0, it = 0;
            if (next[i] >= nsteps[i]) continue;
            st = evpg_job_collect(jobs[i], batch, i, &ended, &it);
            if (st || !ended) continue;
            if (iters) iters[(size_t)i * stride + next[i]] = it;
            next[i]++;
            if (next[i] < nsteps[i]) st = evpg_job_stage(jobs[i], batch, i, next[i]);
            else left--;
        }
    }
    if (rounds_out) *rounds_out = rounds;
    evpg_batch_destroy(batch);
    free(ctxs);
    free(next);
    return st;
}

int evpg_job_scalars(void *jp, double *o, int32_t count)
{
    evpg_job *j = (evpg_job *)jp;
    double s[34];
    if (!j || !o) return EVPG_ERR_ARG;
    s[0] = j->TimeTot; s[1] = j->e_vm; s[2] = j->evmp; s[3] = j->d_vm; s[4] = j->dvmp;
    s[5] = j->s_vm; s[6] = j->s_vm1;
    memcpy(s + 7, j->SigAvg, 72);
    memcpy(s + 16, j->SigAvg1, 72);
    memcpy(s + 25, j->rho_avg, 64);
    s[33] = (double)j->nr_iters;
    memcpy(o, s, sizeof(double) * (size_t)(count < 34 ? count : 34));
    return EVPG_OK;
}

static void wdoubles(const char *dir, const char *name, const double *x, int n)
{
    char p[1200];
    FILE *f;
    snprintf(p, sizeof p, "%s/%s", dir, name);
    f = fopen(p, "wb");
    if (!f) return;
    fwrite(x, sizeof(double), (size_t)n, f);
    fclose(f);
}

/* .iout dumps (io.c:322-995): eps, els, sig (6 files each, order 11,22,33,
 * 23,13,12), rho SSD sum, texture records, slip and dislocation records
 * (int grain + 4 padding + 12 doubles), new_position. */
static int write_iout(evpg_job *j, const char *dir, int step)
{
    const int N = j->N;
    double *sig = (double *)malloc(sizeof(double) * 9 * (size_t)N);
    double *dgr = (double *)malloc(sizeof(double) * 9 * (size_t)N);
    double *eps = (double *)malloc(sizeof(double) * 9 * (size_t)N);
    double *tr = (double *)malloc(sizeof(double) * 9 * (size_t)N);
    double *rs = (double *)malloc(sizeof(double) * 12 * (size_t)N);
    double *ga = (double *)malloc(sizeof(double) * 12 * (size_t)N);
    double *tmp = (double *)malloc(sizeof(double) * (size_t)N);
    static const int ci[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};
    char name[200], p[1200];
    int c, v, i, st = EVPG_ERR_NOMEM;
    unsigned char rec[104];
    FILE *f;
    if (!sig || !dgr || !eps || !tr || !rs || !ga || !tmp) goto done;
    if ((st = evpg_download(j->ctx, EVPG_F_SIG, sig, 9 * (size_t)N))) goto done;
    if ((st = evpg_download(j->ctx, EVPG_F_DISGRAD, dgr, 9 * (size_t)N))) goto done;
    if ((st = evpg_download(j->ctx, EVPG_F_EPS, eps, 9 * (size_t)N))) goto done;
    if ((st = evpg_download(j->ctx, EVPG_F_TRANMAT, tr, 9 * (size_t)N))) goto done;
    if ((st = evpg_download(j->ctx, EVPG_F_RHO_S, rs, 12 * (size_t)N))) goto done;
    if ((st = evpg_download(j->ctx, EVPG_F_GAM_ACUM, ga, 12 * (size_t)N))) goto done;
    for (c = 0; c < 6; c++) {
        const int a = ci[c][0], b = ci[c][1];
        for (v = 0; v < N; v++) tmp[v] = eps[9 * (size_t)v + 3 * a + b];
        snprintf(name, sizeof name, "eps_%01d_S%06d.iout", c + 1, step);
        wdoubles(dir, name, tmp, N);
        for (v = 0; v < N; v++) {
            const double *g = dgr + 9 * (size_t)v;
            tmp[v] = (c < 3) ? g[4 * a] - eps[9 * (size_t)v + 4 * a]
                             : (g[3 * a + b] + g[3 * b + a]) / 2.0 - eps[9 * (size_t)v + 3 * a + b];
        }
        snprintf(name, sizeof name, "els_%01d_S%06d.iout", c + 1, step);
        wdoubles(dir, name, tmp, N);
        for (v = 0; v < N; v++) tmp[v] = sig[9 * (size_t)v + 3 * a + b];
        snprintf(name, sizeof name, "sig_afterDRX_%01d_S%06d.iout", c + 1, step);
        wdoubles(dir, name, tmp, N);
    }
    for (v = 0; v < N; v++) {
        const int p2 = j->phase_f[v] - 1;
        tmp[v] = 0.0;
        for (i = 0; i < j->nSYS[p2]; i++) tmp[v] += rs[12 * (size_t)v + i];
    }
    snprintf(name, sizeof name, "rho_afterDRX_SSD_S%06d.iout", step);
    wdoubles(dir, name, tmp, N);
    snprintf(p, sizeof p, "%s/tex_afterDRX_S%06d.iout", dir, step);
    f = fopen(p, "wb");
    for (v = 0; f && v < N; v++) {
        t2 sa;
        double ang[3];
        int co[6], a, b;
        for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) sa[a][b] = tr[9 * (size_t)v + 3 * b + a];
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
        memcpy(rec + 8, ga + 12 * (size_t)v, 96);
        fwrite(rec, 1, 104, f);
    }
    if (f) fclose(f);
    snprintf(p, sizeof p, "%s/dislocation_afterDRX_S%04d.iout", dir, step);
    f = fopen(p, "wb");
    for (v = 0; f && v < N; v++) {
        memset(rec, 0, sizeof rec);
        memcpy(rec, &j->grain_f[v], 4);
        memcpy(rec + 8, rs + 12 * (size_t)v, 96);
        fwrite(rec, 1, 104, f);
    }
    if (f) fclose(f);
    /* WriteNewPositionMPI (io.c:723-790): new_position + displacement_fluct
     * - x with new_position = (I + DisGrad) x (evolution.c:1434-1438) and
     * displacement_fluct[i] = -fluctuation[i][2] (what evolution.c:1401-1425
     * computes as written). fluctuation = DisGrad minus its uniform part,
     * DisGradAvg_actual less the mixed-BC corrections of each loop's last
     * iteration, which never reached DisGrad. Creep resets DisGrad each
     * increment while the reference's fluctuation keeps accumulating, so that
     * record is written as zeros there. */
    snprintf(p, sizeof p, "%s/new_position_afterDRX_S%04d.iout", dir, step);
    f = fopen(p, "wb");
    for (v = 0; f && v < N; v++) {
        const double *D = dgr + 9 * (size_t)v;
        const double px = (double)(v / (j->n1 * j->n2)), py = (double)((v / j->n2) % j->n1),
                     pz = (double)(v % j->n2);
        double np3[3], ss[3] = {0.0, 0.0, 0.0};
        int a;
        if (j->CREEP_FLAG != 1) {
            np3[0] = (1.0 + D[0]) * px + D[1] * py + D[2] * pz;
            np3[1] = (1.0 + D[4]) * py + D[3] * px + D[5] * pz;
            np3[2] = (1.0 + D[8]) * pz + D[6] * px + D[7] * py;
            for (a = 0; a < 3; a++) {
                const double disp = -(D[3 * a + 2] - (j->DisGradAvg_actual[a][2] - j->dE_unapplied[a][2]));
                ss[a] = np3[a] + disp - (a == 0 ? px : a == 1 ? py : pz);
            }
        }
        fwrite(ss, sizeof(double), 3, f);
    }
    if (f) fclose(f);
    st = EVPG_OK;
done:
    free(sig); free(dgr); free(eps); free(tr); free(rs); free(ga); free(tmp);
    return st;
}

int evpg_job_run(void *jp, const char *outdir, int32_t nsteps, int32_t write_iout_flag)
{
    evpg_job *j = (evpg_job *)jp;
    char p[1200];
    FILE *fvm, *fdd, *ferr, *fit;
    int istep, st = EVPG_OK;
    int32_t it = 0;
    if (!j || !outdir) return EVPG_ERR_ARG;
    if (nsteps < 0) nsteps = j->nl.N_steps;
    snprintf(p, sizeof p, "%s/vm.out", outdir); fvm = fopen(p, "w");
    snprintf(p, sizeof p, "%s/dd.out", outdir); fdd = fopen(p, "w");
    snprintf(p, sizeof p, "%s/err.out", outdir); ferr = fopen(p, "w");
    snprintf(p, sizeof p, "%s/iters.txt", outdir); fit = fopen(p, "w");
    snprintf(p, sizeof p, "%s/errors.txt", outdir); j->err_log = fopen(p, "w");
    if (!fvm || !fdd || !ferr || !fit || !j->err_log) {
        if (fvm) fclose(fvm);
        if (fdd) fclose(fdd);
        if (ferr) fclose(ferr);
        if (fit) fclose(fit);
        if (j->err_log) fclose(j->err_log);
        j->err_log = 0;
        return EVPG_ERR_IO;
    }
    fprintf(fvm, "TIME\tEVM\tEVMP\tDVM\tDVMP\tSVM\tSVMSVM_1\n");
    fprintf(fdd, "TIME\tEVM\tDD_F\tDD_P\tDD_s\tDD_m\tDD_g\n");
    fprintf(ferr, "IT\tERRE\tERRS\tSVM\n");
    for (istep = 0; istep < nsteps; istep++) {
        if (nsteps != 1) fprintf(ferr, "STEP = %d\n", istep);
        if (j->CREEP_FLAG == 1 && j->e_vm > 0.3) break;
        st = evpg_job_increment(j, istep, &it);
        fprintf(fit, "%d %d\n", istep, it);
        if (st) break;
        fprintf(fdd, "%e\t%e\t%e\t%e\t%e\t%e\t%e\n", j->TimeTot, j->e_vm, j->rho_avg[2], j->rho_avg[3],
                j->rho_avg[5], j->rho_avg[7], j->rho_avg[6]);
        fprintf(fvm, "%e\t%e\t%e\t%e\t%e\t%e\t%e\n", j->TimeTot, j->e_vm, j->evmp, j->d_vm, j->dvmp,
                j->s_vm, j->s_vm1);
        if (write_iout_flag && j->nl.PrintControl[0] == 1 && j->nl.PrintControl[1] > 0 &&
            istep % j->nl.PrintControl[1] == 0) {
            st = write_iout(j, outdir, istep);
            if (st) break;
        }
    }
    fclose(fvm); fclose(fdd); fclose(ferr); fclose(fit); fclose(j->err_log);
    j->err_log = 0;
    return st;
}
