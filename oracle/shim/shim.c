/*
 * Single-rank MPI, FFTW 2 MPI and GSL stand-ins (see the headers in this
 * directory). TEST INFRASTRUCTURE ONLY: linked into the oracle/_ref binary.
 */
#include <mpi.h>
#include <fftw_mpi.h>
#include <gsl/gsl_rng.h>
#include <gsl/gsl_randist.h>

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../fft_cpu.h"

/* ------------------------------------------------------------------ MPI */

#define SRX_MAX_TYPES 256
#define SRX_MAX_BLOCKS 32

typedef struct {
    long extent;
    int nblk;
    long disp[SRX_MAX_BLOCKS];
    long size[SRX_MAX_BLOCKS];
} srx_type;

static srx_type g_types[SRX_MAX_TYPES];
static int g_ntypes = 4; /* 0 unused, 1 int, 2 double, 3 float */

static const srx_type *type_get(MPI_Datatype t)
{
    static int init = 0;
    if (!init) {
        g_types[MPI_INT].extent = 4;
        g_types[MPI_INT].nblk = 1; g_types[MPI_INT].disp[0] = 0; g_types[MPI_INT].size[0] = 4;
        g_types[MPI_DOUBLE].extent = 8;
        g_types[MPI_DOUBLE].nblk = 1; g_types[MPI_DOUBLE].disp[0] = 0; g_types[MPI_DOUBLE].size[0] = 8;
        g_types[MPI_FLOAT].extent = 4;
        g_types[MPI_FLOAT].nblk = 1; g_types[MPI_FLOAT].disp[0] = 0; g_types[MPI_FLOAT].size[0] = 4;
        init = 1;
    }
    if (t <= 0 || t >= g_ntypes) {
        fprintf(stderr, "mpi shim: unknown datatype %d\n", t);
        exit(90);
    }
    return &g_types[t];
}

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; type_get(MPI_INT); return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_size(MPI_Comm c, int *size) { (void)c; *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm c, int *rank) { (void)c; *rank = 0; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
int MPI_Abort(MPI_Comm c, int code)
{
    (void)c;
    fprintf(stderr, "MPI_Abort(%d)\n", code);
    fflush(stdout);
    exit(code ? code : 1);
}

int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
    (void)op; (void)c;
    memmove(r, s, (size_t)count * (size_t)type_get(t)->extent);
    return 0;
}

int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt,
                  MPI_Comm c)
{
    (void)rc; (void)rt; (void)c;
    memmove(r, s, (size_t)sc * (size_t)type_get(st)->extent);
    return 0;
}

int MPI_Allgatherv(const void *s, int sc, MPI_Datatype st, void *r, const int *rcounts,
                   const int *displs, MPI_Datatype rt, MPI_Comm c)
{
    (void)rcounts; (void)c;
    if (sc > 0)
        memmove((char *)r + (size_t)displs[0] * (size_t)type_get(rt)->extent, s,
                (size_t)sc * (size_t)type_get(st)->extent);
    return 0;
}

static int p2p_unsupported(const char *what)
{
    fprintf(stderr, "mpi shim: %s is not available with one rank\n", what);
    exit(91);
}

int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{
    (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c;
    return p2p_unsupported("MPI_Send");
}
int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st)
{
    (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st;
    return p2p_unsupported("MPI_Recv");
}
int MPI_Sendrecv(const void *sb, int sc, MPI_Datatype stt, int d, int stag, void *rb, int rc,
                 MPI_Datatype rt, int s, int rtag, MPI_Comm c, MPI_Status *st)
{
    (void)sb; (void)sc; (void)stt; (void)d; (void)stag; (void)rb; (void)rc; (void)rt;
    (void)s; (void)rtag; (void)c; (void)st;
    return p2p_unsupported("MPI_Sendrecv");
}

int MPI_Address(const void *loc, MPI_Aint *addr)
{
    *addr = (MPI_Aint)(size_t)loc;
    return 0;
}

int MPI_Type_struct(int count, const int *blocklens, const MPI_Aint *indices,
                    const MPI_Datatype *types, MPI_Datatype *newtype)
{
    srx_type *nt;
    long ub = 0, align = 1;
    int i;
    if (g_ntypes >= SRX_MAX_TYPES) {
        fprintf(stderr, "mpi shim: too many datatypes\n");
        exit(92);
    }
    nt = &g_types[g_ntypes];
    nt->nblk = 0;
    for (i = 0; i < count; i++) {
        const srx_type *bt = type_get(types[i]);
        long e = bt->extent * blocklens[i];
        if (nt->nblk >= SRX_MAX_BLOCKS) {
            fprintf(stderr, "mpi shim: struct datatype too large\n");
            exit(92);
        }
        nt->disp[nt->nblk] = indices[i];
        nt->size[nt->nblk] = e;
        nt->nblk++;
        if (indices[i] + e > ub) ub = indices[i] + e;
        if (bt->extent > align) align = bt->extent;
    }
    /* MPI pads the extent of a struct type to its strictest member alignment. */
    nt->extent = ((ub + align - 1) / align) * align;
    *newtype = g_ntypes++;
    return 0;
}

int MPI_Type_commit(MPI_Datatype *t) { (void)type_get(*t); return 0; }

struct srx_mpi_file {
    FILE *fp;
    long long disp;
};

int MPI_File_open(MPI_Comm c, const char *fname, int amode, MPI_Info info, MPI_File *fh)
{
    (void)c; (void)amode; (void)info;
    *fh = (MPI_File)calloc(1, sizeof(struct srx_mpi_file));
    (*fh)->fp = fopen(fname, "wb");
    if (!(*fh)->fp) {
        fprintf(stderr, "mpi shim: cannot open %s\n", fname);
        exit(93);
    }
    return 0;
}

int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype et, MPI_Datatype ft,
                      const char *rep, MPI_Info info)
{
    (void)et; (void)ft; (void)rep; (void)info;
    fh->disp = disp;
    return 0;
}

int MPI_File_write(MPI_File fh, const void *buf, int count, MPI_Datatype t, MPI_Status *st)
{
    const srx_type *ty = type_get(t);
    char *rec = (char *)malloc((size_t)ty->extent);
    int i, b;
    (void)st;
    fseek(fh->fp, (long)fh->disp, SEEK_SET);
    for (i = 0; i < count; i++) {
        const char *src = (const char *)buf + (size_t)i * (size_t)ty->extent;
        memset(rec, 0, (size_t)ty->extent);
        for (b = 0; b < ty->nblk; b++)
            memcpy(rec + ty->disp[b], src + ty->disp[b], (size_t)ty->size[b]);
        fwrite(rec, 1, (size_t)ty->extent, fh->fp);
    }
    free(rec);
    return 0;
}

int MPI_File_close(MPI_File *fh)
{
    if (*fh) {
        fclose((*fh)->fp);
        free(*fh);
        *fh = 0;
    }
    return 0;
}

/* ------------------------------------------------------------- FFTW 2 */

struct srx_fftwnd_plan {
    int n[3];
    int sign;
};

fftwnd_mpi_plan fftw3d_mpi_create_plan(MPI_Comm c, int nx, int ny, int nz, fftw_direction dir,
                                       int flags)
{
    fftwnd_mpi_plan p = (fftwnd_mpi_plan)calloc(1, sizeof(*p));
    (void)c; (void)flags;
    p->n[0] = nx;
    p->n[1] = ny;
    p->n[2] = nz;
    p->sign = (dir == FFTW_FORWARD) ? -1 : 1;
    return p;
}

void fftwnd_mpi_local_sizes(fftwnd_mpi_plan p, int *lnx, int *lxs, int *lnyt, int *lyst,
                            int *lsize)
{
    *lnx = p->n[0];
    *lxs = 0;
    *lnyt = p->n[1];
    *lyst = 0;
    *lsize = p->n[0] * p->n[1] * p->n[2];
}

void fftwnd_mpi(fftwnd_mpi_plan p, int n_fields, fftw_complex *data, fftw_complex *work,
                fftwnd_mpi_output_order order)
{
    (void)work; (void)order;
    if (n_fields != 1 || srx_fft3d((double *)data, p->n[0], p->n[1], p->n[2], p->sign)) {
        fprintf(stderr, "fftw shim: unsupported transform\n");
        exit(94);
    }
}

void fftwnd_mpi_destroy_plan(fftwnd_mpi_plan p) { free(p); }

void *fftw_malloc(size_t n)
{
    /* Twice the request plus a margin, zero-filled (see fftw_mpi.h). */
    return calloc(2 * n + 4096, 1);
}

void fftw_free(void *p) { free(p); }

/* ---------------------------------------------------------------- GSL */

static const gsl_rng_type g_default_type = {"srx-shim"};
const gsl_rng_type *gsl_rng_default = &g_default_type;
unsigned long gsl_rng_default_seed = 0;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T)
{
    gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
    (void)T;
    r->state = 0x9E3779B97F4A7C15ull;
    return r;
}

void gsl_rng_free(gsl_rng *r) { free(r); }

double gsl_rng_uniform(const gsl_rng *r)
{
    gsl_rng *m = (gsl_rng *)r;
    m->state = m->state * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(m->state >> 11) * (1.0 / 9007199254740992.0);
}

double gsl_ran_weibull(const gsl_rng *r, double a, double b)
{
    (void)b;
    return a * gsl_rng_uniform(r);
}
