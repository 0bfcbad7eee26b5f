/*
 * Harness around the reference's own sources (TEST INFRASTRUCTURE ONLY).
 *
 * Built by oracle/Makefile into oracle/_ref/srx_ref from the unmodified files
 * under the reference tree (io.c, init.c, kinematics.c, constitutive.c, and
 * evolution.c, which is included below so that its static UpdateStress() and
 * get_smacro() can be driven directly). It replaces the reference main
 * (evp.c:7-32) with the same call sequence plus hooks:
 *
 *   srx_ref <input> [--rho0 FILE] [--final FILE]
 *       GetNameList, MPI_Init, PrintNameList, OpenFiles, SetupJob,
 *       [per-voxel initial SSD density from FILE: N doubles, 1e12 m^-2,
 *        the same value on every slip system], Evolution,
 *       [final state dump, GND densities last], DestroyJob, CloseFiles.
 *
 *   srx_ref <input> --setup FILE
 *       SetupJob, update_schmid() (as the first increment does,
 *       evolution.c:1130-1132), then dump the set-up state.
 *
 *   srx_ref <input> --nr IN OUT
 *       SetupJob, update_schmid(), read Sig/DisGrad/Eps/rho_s/rho_m from IN,
 *       run one UpdateStress() sweep (evolution.c:157-427) and dump
 *       Sig/Edot/rho_m/gamdot/trial_gam_acum/rho_F/rho_P and the error sums.
 *
 * Binary formats are little-endian doubles in the reference's own AoS voxel
 * order (pIDX, evp.h:60), written by the functions below.
 */
#define EVP_GLOBALS_ONCE
#include "evp.h"
#undef EVP_GLOBALS_ONCE
#include "evolution.c"

#include <string>

static void put(FILE *f, const void *p, size_t n) { fwrite(p, 1, n, f); }

static void put_t2(FILE *f, ten2nd *a) { put(f, a, sizeof(ten2nd) * (size_t)lsize); }

static void put_sys(FILE *f, real **a)
{
    for (int v = 0; v < lsize; v++) put(f, a[v], sizeof(real) * NSYSMX);
}

static void get(FILE *f, void *p, size_t n)
{
    if (fread(p, 1, n, f) != n) {
        fprintf(stderr, "srx_ref: short read\n");
        exit(97);
    }
}

static void get_sys(FILE *f, real **a)
{
    for (int v = 0; v < lsize; v++) get(f, a[v], sizeof(real) * NSYSMX);
}

static void load_rho0(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "srx_ref: cannot open %s\n", path); exit(96); }
    for (int v = 0; v < lsize; v++) {
        double r;
        get(f, &r, sizeof r);
        for (int i = 0; i < NSYSMX; i++) {
            rho_s[v][i] = r;
            trial_rho_s[v][i] = r;
        }
    }
    fclose(f);
}

static void dump_final(const char *path)
{
    FILE *f = fopen(path, "wb");
    int hdr[2] = {lsize, NSYSMX};
    put(f, hdr, sizeof hdr);
    put_t2(f, Sig); put_t2(f, DisGrad); put_t2(f, Eps); put_t2(f, Edot);
    put_t2(f, VelGrad); put_t2(f, TranMat_xt2sa);
    put_sys(f, rho_s); put_sys(f, rho_m); put_sys(f, rho_F); put_sys(f, rho_P);
    put_sys(f, gamdot); put_sys(f, gam_acum); put_sys(f, trial_gam_acum);
    put_sys(f, rho_dipole); put_sys(f, rho_forest); put_sys(f, rho_inplane);
    put(f, rho_tot, sizeof(real) * (size_t)lsize);
    put(f, SigAvg, sizeof SigAvg); put(f, SigAvg1, sizeof SigAvg1);
    put(f, dDisGradAvg_acum, sizeof dDisGradAvg_acum); put(f, DisGradAvg, sizeof DisGradAvg);
    double sc[13] = {e_vm, d_vm, s_vm, s_vm1, TimeTot, rho_F_avg, rho_P_avg, rho_s_avg,
                     rho_m_avg, rho_g_avg, rho_dipole_avg, rho_forest_avg, rho_inplane_avg};
    put(f, sc, sizeof sc);
    /* GND densities (zero unless built with DD_GND) */
    put_sys(f, rho_g1); put_sys(f, rho_g2); put_sys(f, rho_g3);
    fclose(f);
}

static void dump_setup(const char *path)
{
    FILE *f = fopen(path, "wb");
    int hdr[2] = {lsize, NSYSMX};
    put(f, hdr, sizeof hdr);
    put(f, C066, sizeof C066); put(f, S066, sizeof S066);
    put(f, C_gr, sizeof(voigt66) * (size_t)lsize);
    put(f, Schm_xt, sizeof Schm_xt);
    put(f, Schm_gr, sizeof(voigtch) * (size_t)lsize);
    for (int i = 0; i < NSYSMX; i++) put(f, Chi[0][i], sizeof(real) * NSYSMX);
    for (int i = 0; i < NSYSMX; i++) put(f, Chi_1[0][i], sizeof(real) * NSYSMX);
    put(f, Shear_G, sizeof Shear_G);
    put(f, bb_B, sizeof bb_B);
    put_t2(f, TranMat_xt2sa);
    put_t2(f, Sig);
    double sc[4] = {d_vm, e_vm, WGT, Wgt_ph1};
    put(f, sc, sizeof sc);
    put(f, S0, sizeof S0);
    put(f, B, sizeof B);
    fclose(f);
}

static void nr_probe(const char *in, const char *out)
{
    FILE *f = fopen(in, "rb");
    if (!f) { fprintf(stderr, "srx_ref: cannot open %s\n", in); exit(96); }
    get(f, Sig, sizeof(ten2nd) * (size_t)lsize);
    get(f, DisGrad, sizeof(ten2nd) * (size_t)lsize);
    get(f, Eps, sizeof(ten2nd) * (size_t)lsize);
    get_sys(f, rho_s);
    get_sys(f, rho_m);
    fclose(f);
    for (int v = 0; v < lsize; v++)
        for (int i = 0; i < NSYSMX; i++) trial_rho_s[v][i] = rho_s[v][i];
    real err_e = 0.0, err_s = 0.0;
    UpdateStress(0, &err_e, &err_s, 1);
    f = fopen(out, "wb");
    put_t2(f, Sig); put_t2(f, Edot);
    put_sys(f, rho_m); put_sys(f, gamdot); put_sys(f, trial_gam_acum);
    put_sys(f, rho_F); put_sys(f, rho_P);
    double sc[2] = {err_e, err_s};
    put(f, sc, sizeof sc);
    fclose(f);
}

int main(int argc, char **argv)
{
    const char *rho0 = 0, *final_path = 0, *setup_path = 0, *nr_in = 0, *nr_out = 0;
    if (argc < 2) {
        fprintf(stderr, "usage: srx_ref <input> [--rho0 F] [--final F] [--setup F] [--nr IN OUT]\n");
        return 2;
    }
    for (int a = 2; a < argc; a++) {
        std::string s = argv[a];
        if (s == "--rho0" && a + 1 < argc) rho0 = argv[++a];
        else if (s == "--final" && a + 1 < argc) final_path = argv[++a];
        else if (s == "--setup" && a + 1 < argc) setup_path = argv[++a];
        else if (s == "--nr" && a + 2 < argc) { nr_in = argv[++a]; nr_out = argv[++a]; }
        else { fprintf(stderr, "srx_ref: bad argument %s\n", argv[a]); return 2; }
    }
    GetNameList(argv);
    MPI_Init(&argc, &argv);
    MPI_Comm_size(MPI_COMM_WORLD, &NumPE);
    MPI_Comm_rank(MPI_COMM_WORLD, &mpirank);
    PrintNameList();
    OpenFiles();
    SetupJob();
    if (rho0) load_rho0(rho0);
    if (setup_path || nr_in) {
        update_schmid();
        if (setup_path) dump_setup(setup_path);
        if (nr_in) nr_probe(nr_in, nr_out);
    } else {
        Evolution();
        if (final_path) dump_final(final_path);
    }
    DestroyJob();
    CloseFiles();
    MPI_Finalize();
    return 0;
}
