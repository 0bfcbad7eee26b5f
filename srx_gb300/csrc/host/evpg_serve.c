/*
 * evpg_serve.c -- continuous-batching server for EVP-FFT solves.
 *
 * Requests (a namelist file, optional per-voxel initial density, an increment
 * count and an optional load switch) arrive at any time through
 * evpg_server_submit. Loader threads open them -- parse the input files, set
 * up the RVE, upload it -- as soon as the device-memory budget allows
 * (admission by the footprint evpg_estimate_bytes reports, FIFO order). One
 * GPU thread owns a batch: between rounds it admits opened requests into free
 * slots, stages every slot's next increment, runs one round (at most
 * round_ticks equilibrium iterations of all running RVEs, one CUDA graph),
 * finishes the increments that ended, applies load switches, and retires
 * finished solves (their device memory returns to the budget). So a request
 * that arrives while others run starts at the next round boundary and its
 * work shares the same kernel launches as theirs; each RVE's arithmetic is
 * the same as alone.
 *
 * No counterpart in the reference (one RVE per MPI job, evp.c:7-32).
 */
#define _POSIX_C_SOURCE 200809L
#include "evpg.h"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

enum { RQ_QUEUED = 0, RQ_LOADING = 1, RQ_READY = 2, RQ_RUNNING = 3, RQ_DONE = 4, RQ_FAILED = 5 };

typedef struct req {
    int64_t id;
    char input[1024], rho0[1024], sw_input[1024];
    int nsteps, switch_step, state, status;
    double t_submit, t_admit, t_done, t_incr;
    int incr_done, need_stage;
    long long iters;
    int64_t bytes;
    void *job;
    double *sig6, *rho_s, scalars[34];   /* kept results (cfg.keep_fields) */
    int nvox;
} req;

typedef struct server {
    evpg_server_cfg cfg;
    pthread_mutex_t mu;
    pthread_cond_t cv_load, cv_gpu, cv_done;
    req **all;
    int nall, capall;
    int next_pending;          /* FIFO cursor over all[] */
    req **ready;
    int nready, capready;
    int loading;
    int64_t used;
    req **act;
    int nact;
    double *lat;
    int nlat, caplat;
    long long rounds, ticks;
    int shutdown, gpu_error;
    double t0;
    pthread_t gpu;
    pthread_t *loaders;
    void *batch;
} server;

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void push_lat(server *s, double v)
{
    if (s->nlat == s->caplat) {
        int cap = s->caplat ? 2 * s->caplat : 1024;
        double *p = (double *)realloc(s->lat, sizeof(double) * (size_t)cap);
        if (!p) return;
        s->lat = p;
        s->caplat = cap;
    }
    s->lat[s->nlat++] = v;
}

static void *loader_main(void *arg)
{
    server *s = (server *)arg;
    pthread_mutex_lock(&s->mu);
    for (;;) {
        req *r;
        int32_t n[3];
        int64_t bytes = 0;
        int st;
        while (!s->shutdown && s->next_pending >= s->nall) pthread_cond_wait(&s->cv_load, &s->mu);
        if (s->shutdown) break;
        r = s->all[s->next_pending++];
        s->loading++;
        pthread_mutex_unlock(&s->mu);
        st = evpg_job_grid(r->input, n);
        if (!st) st = evpg_estimate_bytes(n, s->cfg.precision, 0, &bytes);
        /* GND densities: 24 doubles and one byte per voxel */
        if (!st && (s->cfg.job_options & EVPG_JOB_GND)) bytes += 193LL * n[0] * n[1] * n[2];
        /* orientation rows and allocator granularity */
        bytes += bytes / 16 + (16 << 20);
        pthread_mutex_lock(&s->mu);
        if (!st && bytes > s->cfg.hbm_budget) st = EVPG_ERR_NOMEM;
        while (!st && !s->shutdown && s->used + bytes > s->cfg.hbm_budget) pthread_cond_wait(&s->cv_load, &s->mu);
        if (s->shutdown) { s->loading--; break; }
        if (!st) {
            s->used += bytes;
            r->bytes = bytes;
            r->state = RQ_LOADING;
            pthread_mutex_unlock(&s->mu);
            st = evpg_job_open_opts(r->input, r->rho0[0] ? r->rho0 : NULL, s->cfg.precision, s->cfg.nr_mode,
                                    s->cfg.job_options, &r->job);
            pthread_mutex_lock(&s->mu);
        }
        s->loading--;
        if (st) {
            r->state = RQ_FAILED;
            r->status = st;
            r->t_done = now_s();
            s->used -= r->bytes;
            r->bytes = 0;
            pthread_cond_broadcast(&s->cv_done);
            pthread_cond_broadcast(&s->cv_load);
            continue;
        }
        if (s->nready == s->capready) {
            int cap = s->capready ? 2 * s->capready : 64;
            req **p = (req **)realloc(s->ready, sizeof(req *) * (size_t)cap);
            if (p) { s->ready = p; s->capready = cap; }
        }
        r->state = RQ_READY;
        s->ready[s->nready++] = r;
        pthread_cond_signal(&s->cv_gpu);
    }
    pthread_mutex_unlock(&s->mu);
    return NULL;
}

/* Slots = the active requests in order; re-stage every request that waits
 * for its next increment (staging is per slot index). */
static int compose(server *s)
{
    void **ctxs = (void **)calloc((size_t)(s->nact > 0 ? s->nact : 1), sizeof(void *));
    int i, st;
    for (i = 0; i < s->nact; i++) ctxs[i] = evpg_job_ctx(s->act[i]->job);
    st = evpg_batch_set(s->batch, ctxs, s->nact);
    free(ctxs);
    return st;
}

static void finish_req(server *s, req *r, int state, int status)
{
    if (state == RQ_DONE && s->cfg.keep_fields) {
        int32_t n[3];
        if (!evpg_job_nvox(r->job, n)) {
            const size_t N = (size_t)n[0] * n[1] * n[2];
            r->sig6 = (double *)malloc(sizeof(double) * 6 * N);
            r->rho_s = (double *)malloc(sizeof(double) * 12 * N);
            if (r->sig6 && r->rho_s) {
                void *c = evpg_job_ctx(r->job);
                if (evpg_download(c, EVPG_F_SIG6, r->sig6, 6 * N) || evpg_download(c, EVPG_F_RHO_S, r->rho_s, 12 * N))
                    status = EVPG_ERR_CUDA;
                evpg_job_scalars(r->job, r->scalars, 34);
                r->nvox = (int)N;
            }
        }
    }
    evpg_job_close(r->job);
    r->job = NULL;
    pthread_mutex_lock(&s->mu);
    r->state = state;
    r->status = status;
    r->t_done = now_s();
    s->used -= r->bytes;
    r->bytes = 0;
    pthread_cond_broadcast(&s->cv_load);
    pthread_cond_broadcast(&s->cv_done);
    pthread_mutex_unlock(&s->mu);
}

static void *gpu_main(void *arg)
{
    server *s = (server *)arg;
    int st = evpg_batch_create(s->cfg.precision, s->cfg.nr_mode, &s->batch);
    if (st) {
        pthread_mutex_lock(&s->mu);
        s->gpu_error = st;
        pthread_cond_broadcast(&s->cv_done);
        pthread_mutex_unlock(&s->mu);
        return NULL;
    }
    for (;;) {
        int changed = 0, i, k;
        int32_t ticks = 0;
        double t;
        pthread_mutex_lock(&s->mu);
        while (!s->shutdown && s->nact == 0 && s->nready == 0) pthread_cond_wait(&s->cv_gpu, &s->mu);
        if (s->shutdown) {
            pthread_mutex_unlock(&s->mu);
            break;
        }
        t = now_s();
        while (s->nready > 0 && s->nact < s->cfg.max_slots) {
            req *r = s->ready[0];
            memmove(s->ready, s->ready + 1, sizeof(req *) * (size_t)(s->nready - 1));
            s->nready--;
            r->state = RQ_RUNNING;
            r->t_admit = t;
            r->need_stage = 1;
            s->act[s->nact++] = r;
            changed = 1;
        }
        pthread_mutex_unlock(&s->mu);
        if (changed && (st = compose(s)) != 0) break;
        t = now_s();
        for (i = 0; i < s->nact && !st; i++) {
            req *r = s->act[i];
            if (!r->need_stage) continue;
            st = evpg_job_stage(r->job, s->batch, i, r->incr_done);
            r->need_stage = 0;
            r->t_incr = t;
        }
        if (st) break;
        st = evpg_batch_round(s->batch, s->cfg.round_ticks, &ticks);
        if (st) break;
        t = now_s();
        s->rounds++;
        s->ticks += ticks;
        k = 0;
        changed = 0;
        for (i = 0; i < s->nact; i++) {
            req *r = s->act[i];
            int32_t ended = 0, it = 0;
            int cst = evpg_job_collect(r->job, s->batch, i, &ended, &it);
            if (cst) {
                finish_req(s, r, RQ_FAILED, cst);
                changed = 1;
                continue;
            }
            if (ended) {
                pthread_mutex_lock(&s->mu);
                push_lat(s, t - r->t_incr);
                pthread_mutex_unlock(&s->mu);
                r->incr_done++;
                r->iters += it;
                if (r->switch_step > 0 && r->incr_done == r->switch_step && r->sw_input[0]) {
                    cst = evpg_job_set_load_from(r->job, r->sw_input);
                    if (cst) {
                        finish_req(s, r, RQ_FAILED, cst);
                        changed = 1;
                        continue;
                    }
                }
                if (r->incr_done >= r->nsteps) {
                    finish_req(s, r, RQ_DONE, 0);
                    changed = 1;
                    continue;
                }
                r->need_stage = 1;
            }
            s->act[k++] = r;
        }
        s->nact = k;
        if (changed && (st = compose(s)) != 0) break;
    }
    if (st) {
        int i;
        pthread_mutex_lock(&s->mu);
        s->gpu_error = st;
        pthread_mutex_unlock(&s->mu);
        for (i = 0; i < s->nact; i++) finish_req(s, s->act[i], RQ_FAILED, st);
        s->nact = 0;
    }
    evpg_batch_destroy(s->batch);
    s->batch = NULL;
    return NULL;
}

int evpg_server_create(const evpg_server_cfg *cfg, void **out)
{
    server *s;
    int i;
    if (!cfg || !out || cfg->max_slots < 1 || cfg->round_ticks < 1 || cfg->hbm_budget <= 0) return EVPG_ERR_ARG;
    *out = NULL;
    s = (server *)calloc(1, sizeof(server));
    if (!s) return EVPG_ERR_NOMEM;
    s->cfg = *cfg;
    if (s->cfg.loaders < 1) s->cfg.loaders = 1;
    s->act = (req **)calloc((size_t)cfg->max_slots, sizeof(req *));
    s->loaders = (pthread_t *)calloc((size_t)s->cfg.loaders, sizeof(pthread_t));
    pthread_mutex_init(&s->mu, NULL);
    pthread_cond_init(&s->cv_load, NULL);
    pthread_cond_init(&s->cv_gpu, NULL);
    pthread_cond_init(&s->cv_done, NULL);
    s->t0 = now_s();
    if (pthread_create(&s->gpu, NULL, gpu_main, s)) return EVPG_ERR_NOMEM;
    for (i = 0; i < s->cfg.loaders; i++) pthread_create(&s->loaders[i], NULL, loader_main, s);
    *out = s;
    return EVPG_OK;
}

int evpg_server_submit(void *sp, const char *input, const char *rho0, int32_t nsteps, int32_t switch_step,
                       const char *switch_input, int64_t *id)
{
    server *s = (server *)sp;
    req *r;
    if (!s || !input || nsteps < 1) return EVPG_ERR_ARG;
    r = (req *)calloc(1, sizeof(req));
    if (!r) return EVPG_ERR_NOMEM;
    snprintf(r->input, sizeof r->input, "%s", input);
    if (rho0) snprintf(r->rho0, sizeof r->rho0, "%s", rho0);
    if (switch_input) snprintf(r->sw_input, sizeof r->sw_input, "%s", switch_input);
    r->nsteps = nsteps;
    r->switch_step = switch_step;
    r->t_submit = now_s();
    pthread_mutex_lock(&s->mu);
    if (s->nall == s->capall) {
        int cap = s->capall ? 2 * s->capall : 256;
        req **p = (req **)realloc(s->all, sizeof(req *) * (size_t)cap);
        if (!p) { pthread_mutex_unlock(&s->mu); free(r); return EVPG_ERR_NOMEM; }
        s->all = p;
        s->capall = cap;
    }
    r->id = s->nall;
    s->all[s->nall++] = r;
    if (id) *id = r->id;
    pthread_cond_signal(&s->cv_load);
    pthread_mutex_unlock(&s->mu);
    return EVPG_OK;
}

static int all_finished(const server *s)
{
    int i;
    for (i = 0; i < s->nall; i++)
        if (s->all[i]->state != RQ_DONE && s->all[i]->state != RQ_FAILED) return 0;
    return 1;
}

int evpg_server_wait(void *sp, double timeout_s)
{
    server *s = (server *)sp;
    struct timespec ts;
    int rc = EVPG_OK;
    if (!s) return EVPG_ERR_ARG;
    clock_gettime(CLOCK_REALTIME, &ts);
    ts.tv_sec += (time_t)timeout_s;
    ts.tv_nsec += (long)((timeout_s - (double)(time_t)timeout_s) * 1e9);
    if (ts.tv_nsec >= 1000000000L) { ts.tv_sec++; ts.tv_nsec -= 1000000000L; }
    pthread_mutex_lock(&s->mu);
    while (!all_finished(s) && !s->gpu_error) {
        if (pthread_cond_timedwait(&s->cv_done, &s->mu, &ts)) { rc = EVPG_ERR_ITERMAX; break; }
    }
    if (s->gpu_error) rc = s->gpu_error;
    pthread_mutex_unlock(&s->mu);
    return rc;
}

int evpg_server_request(void *sp, int64_t id, evpg_request_info *o)
{
    server *s = (server *)sp;
    req *r;
    if (!s || !o) return EVPG_ERR_ARG;
    pthread_mutex_lock(&s->mu);
    if (id < 0 || id >= s->nall) { pthread_mutex_unlock(&s->mu); return EVPG_ERR_ARG; }
    r = s->all[id];
    o->state = r->state;
    o->status = r->status;
    o->increments = r->incr_done;
    o->iterations = r->iters;
    o->t_submit = r->t_submit - s->t0;
    o->t_admit = r->t_admit > 0 ? r->t_admit - s->t0 : -1.0;
    o->t_done = r->t_done > 0 ? r->t_done - s->t0 : -1.0;
    o->device_bytes = r->bytes;
    pthread_mutex_unlock(&s->mu);
    return EVPG_OK;
}

int evpg_server_result(void *sp, int64_t id, double *sig6, double *rho_s, size_t nvox, double *scalars)
{
    server *s = (server *)sp;
    req *r;
    int st = EVPG_OK;
    if (!s) return EVPG_ERR_ARG;
    pthread_mutex_lock(&s->mu);
    if (id < 0 || id >= s->nall) { pthread_mutex_unlock(&s->mu); return EVPG_ERR_ARG; }
    r = s->all[id];
    if (r->state != RQ_DONE || !r->sig6 || (size_t)r->nvox != nvox) st = EVPG_ERR_ARG;
    else {
        if (sig6) memcpy(sig6, r->sig6, sizeof(double) * 6 * nvox);
        if (rho_s) memcpy(rho_s, r->rho_s, sizeof(double) * 12 * nvox);
        if (scalars) memcpy(scalars, r->scalars, sizeof r->scalars);
    }
    pthread_mutex_unlock(&s->mu);
    return st;
}

static int cmpd(const void *a, const void *b)
{
    const double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

static double pct(const double *v, int n, double p)
{
    double r;
    int i;
    if (n == 0) return 0.0;
    r = p * (double)(n - 1);
    i = (int)r;
    if (i >= n - 1) return v[n - 1];
    return v[i] + (r - (double)i) * (v[i + 1] - v[i]);
}

int evpg_server_stats(void *sp, evpg_serve_stats *o)
{
    server *s = (server *)sp;
    double *sol, *inc, first = 1e300, last = -1e300;
    int i, ns = 0;
    if (!s || !o) return EVPG_ERR_ARG;
    memset(o, 0, sizeof *o);
    pthread_mutex_lock(&s->mu);
    sol = (double *)malloc(sizeof(double) * (size_t)(s->nall + 1));
    inc = (double *)malloc(sizeof(double) * (size_t)(s->nlat + 1));
    for (i = 0; i < s->nall; i++) {
        const req *r = s->all[i];
        if (r->t_submit < first) first = r->t_submit;
        if (r->state == RQ_DONE) {
            sol[ns++] = r->t_done - r->t_submit;
            if (r->t_done > last) last = r->t_done;
            o->increments += r->incr_done;
            o->iterations += r->iters;
        } else if (r->state == RQ_FAILED) {
            o->failed++;
        }
    }
    memcpy(inc, s->lat, sizeof(double) * (size_t)s->nlat);
    o->completed = ns;
    o->rounds = s->rounds;
    o->ticks = s->ticks;
    qsort(sol, (size_t)ns, sizeof(double), cmpd);
    qsort(inc, (size_t)s->nlat, sizeof(double), cmpd);
    o->solve_p50 = pct(sol, ns, 0.50);
    o->solve_p99 = pct(sol, ns, 0.99);
    o->incr_p50 = pct(inc, s->nlat, 0.50);
    o->incr_p99 = pct(inc, s->nlat, 0.99);
    o->span = (ns > 0) ? last - first : 0.0;
    o->solves_per_s = (o->span > 0) ? ns / o->span : 0.0;
    pthread_mutex_unlock(&s->mu);
    free(sol);
    free(inc);
    return EVPG_OK;
}

int evpg_server_destroy(void *sp)
{
    server *s = (server *)sp;
    int i;
    if (!s) return EVPG_OK;
    pthread_mutex_lock(&s->mu);
    s->shutdown = 1;
    pthread_cond_broadcast(&s->cv_load);
    pthread_cond_broadcast(&s->cv_gpu);
    pthread_mutex_unlock(&s->mu);
    pthread_join(s->gpu, NULL);
    for (i = 0; i < s->cfg.loaders; i++) pthread_join(s->loaders[i], NULL);
    for (i = 0; i < s->nact; i++)
        if (s->act[i]->job) evpg_job_close(s->act[i]->job);
    for (i = 0; i < s->nready; i++)
        if (s->ready[i]->job) evpg_job_close(s->ready[i]->job);
    for (i = 0; i < s->nall; i++) {
        free(s->all[i]->sig6);
        free(s->all[i]->rho_s);
        free(s->all[i]);
    }
    free(s->all);
    free(s->ready);
    free(s->act);
    free(s->lat);
    free(s->loaders);
    pthread_mutex_destroy(&s->mu);
    pthread_cond_destroy(&s->cv_load);
    pthread_cond_destroy(&s->cv_gpu);
    pthread_cond_destroy(&s->cv_done);
    free(s);
    return EVPG_OK;
}
