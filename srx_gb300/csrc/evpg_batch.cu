// Batches of RVE contexts advanced together, and the CUDA graph of one
// "round": the increment heads of the RVEs that asked for a new increment,
// then equilibrium iterations over every RVE whose loop is still running
// (one launch per kernel over all RVEs), each RVE's increment tail running
// in the iteration where its loop converges. The iterations sit in a
// conditional WHILE node whose condition a device kernel sets after every
// iteration: the round ends when no RVE is running or after max_ticks
// iterations, without a host round trip.
//
// A batch of one context uses the single-RVE kernels (arguments by value);
// larger batches use the batched kernels, which read each RVE's arguments
// from device tables and map every CTA to (RVE, CTA index within that RVE).
#include "evpg.h"
#include "evpg_ctx.h"

#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <vector>

namespace evpg {

static int bfail(int st, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    return record_error(st, msg);
}

#define BCK(call)                                                                        \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return bfail(EVPG_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                         __FILE__, __LINE__);                                            \
    } while (0)

constexpr int ADVANCE_THREADS = 256;

// Prologue of a round: RVEs whose head just ran start iterating; the WHILE
// condition starts as "some RVE is running".
__global__ void __launch_bounds__(ADVANCE_THREADS) k_round_start(Macro* const* __restrict__ ms, int n,
                                                                 int* tick, const int* kmax,
                                                                 cudaGraphConditionalHandle h) {
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        Macro* m = ms[i];
        if (m->ctl.phase == PH_BEGIN) m->ctl.phase = PH_RUNNING;
        if (m->ctl.phase == PH_RUNNING && !m->done) any = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *tick = 0;
        tick[2] = 0;
        cudaGraphSetConditional(h, (any && *kmax > 0) ? 1u : 0u);
    }
}

// After the macro update of an iteration: the increment-tail section of the
// iteration (an IF node: fold, FP64 refinement, tail, each gated per RVE)
// runs only when some RVE's loop ended in this iteration; tick[2] counts the
// iterations in which it ran.
__global__ void __launch_bounds__(ADVANCE_THREADS) k_if_ending(Macro* const* __restrict__ ms, int n, int* tick,
                                                               cudaGraphConditionalHandle h) {
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (gate_open(ms[i], GATE_ENDING)) any = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        if (any) tick[2] += 1;
        cudaGraphSetConditional(h, any ? 1u : 0u);
    }
}

// End of one iteration: RVEs whose loop finished (and whose tail ran in this
// iteration) are marked ended; the loop continues while some RVE is running
// and fewer than kmax iterations ran in this round.
__global__ void __launch_bounds__(ADVANCE_THREADS) k_advance(Macro* const* __restrict__ ms, int n, int* tick,
                                                             const int* kmax, cudaGraphConditionalHandle h) {
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        Macro* m = ms[i];
        if (m->ctl.phase == PH_RUNNING) {
            if (m->done) m->ctl.phase = PH_ENDED;
            else any = 1;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int t = *tick + 1;
        *tick = t;
        cudaGraphSetConditional(h, (any && t < *kmax) ? 1u : 0u);
    }
}

struct Batch {
    int precision = 0, nr_mode = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // the macro update runs on a side branch of the round graph, beside the
    // next iteration's forward transforms (captured through these)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::vector<Ctx*> slots;
    std::vector<long long> versions;
    bool dirty = true;
    void* dtab[BL_COUNT] = {};
    int2* dmap[BL_COUNT] = {};
    BatchLaunch L[BL_COUNT] = {};
    int* dtk = nullptr;        // [0] tick, [1] kmax, [2] iterations that ran the tail section
    int* htk = nullptr;        // pinned mirror
    IncrCtl* hctl = nullptr;   // pinned, one per slot
    std::vector<char> staged;
    int cap = 0;               // capacity of hctl
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int prologue_kernels = 0, body_kernels = 0, tail_kernels = 0;
    long long launches = 0;
    long long rounds = 0;
};

static void free_tables(Batch& b) {
    for (int k = 0; k < BL_COUNT; k++) {
        if (b.dtab[k]) cudaFree(b.dtab[k]);
        if (b.dmap[k]) cudaFree(b.dmap[k]);
        b.dtab[k] = nullptr;
        b.dmap[k] = nullptr;
        memset(&b.L[k], 0, sizeof(BatchLaunch));
    }
}

static void free_graph(Batch& b) {
    if (b.exec) cudaGraphExecDestroy(b.exec);
    if (b.graph) cudaGraphDestroy(b.graph);
    b.exec = nullptr;
    b.graph = nullptr;
}

// Upload one table: per-slot argument structs + the CTA map.
template <typename A>
static cudaError_t put_table(Batch& b, int kind, const std::vector<A>& args, const std::vector<int>& grids,
                             size_t smem) {
    if (args.empty()) {
        memset(&b.L[kind], 0, sizeof(BatchLaunch));
        return cudaSuccess;
    }
    std::vector<int2> map;
    for (size_t i = 0; i < args.size(); i++)
        for (int q = 0; q < grids[i]; q++) map.push_back(make_int2((int)i, q));
    cudaError_t e = cudaSuccess;
    if (!b.dtab[kind]) e = cudaMalloc(&b.dtab[kind], sizeof(A) * args.size());
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.dtab[kind], args.data(), sizeof(A) * args.size(),
                                              cudaMemcpyHostToDevice, b.stream);
    if (e == cudaSuccess && !map.empty()) {
        if (!b.dmap[kind]) e = cudaMalloc((void**)&b.dmap[kind], sizeof(int2) * map.size());
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(b.dmap[kind], map.data(), sizeof(int2) * map.size(), cudaMemcpyHostToDevice,
                                b.stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b.stream);
    b.L[kind].tab = b.dtab[kind];
    b.L[kind].map = b.dmap[kind];
    b.L[kind].nblk = (int)map.size();
    b.L[kind].smem = smem;
    return e;
}

template <typename T> static const SpecSet<T>& sset(const Ctx& c);
template <> const SpecSet<double>& sset<double>(const Ctx& c) { return c.ks->s64; }
template <> const SpecSet<float>& sset<float>(const Ctx& c) { return c.ks->s32; }
template <typename T> static const NrSet<T>& nrloop(const Ctx& c);
template <> const NrSet<double>& nrloop<double>(const Ctx& c) { return c.ks->nr64; }
template <> const NrSet<float>& nrloop<float>(const Ctx& c) { return c.ks->nr32; }

template <typename T>
static cudaError_t build_tables_t(Batch& b) {
    const size_t n = b.slots.size();
    cudaError_t e = cudaSuccess;
    {
        std::vector<ZArgs<T>> z;
        std::vector<YArgs<T>> yf, yi;
        std::vector<XArgs<T>> x, xw[3];
        std::vector<int> gz, gy, gx, gxw[3];
        size_t smz = 0, smy = 0, smx = 0, smxw[3] = {0, 0, 0};
        // every slot runs the spectral variant it runs alone: the fused z+y
        // plane kernels (one table per lane layout) or the separate passes
        std::vector<PlaneArgs<T>> pa[3];
        std::vector<int> gf[3], gi[3];
        size_t smp[3] = {0, 0, 0};
        // end-of-increment flush of the slots that defer the antisymmetric part
        std::vector<XArgs<T>> xfl[3];
        std::vector<PlaneArgs<T>> pfl[3];
        std::vector<int> gxfl[3], gpfl[3];
        size_t smxfl[3] = {0, 0, 0}, smpfl[3] = {0, 0, 0};
        for (Ctx* c : b.slots) {
            const SpecSet<T>& s = sset<T>(*c);
            if (s.defer) {
                const int q = s.xw == 1 ? 0 : s.xw == 2 ? 1 : 2;
                xfl[q].push_back(s.xfl);
                xfl[q].back().gate = GATE_ENDING;
                gxfl[q].push_back(s.grid_xw);
                if (s.sm_xw > smxfl[q]) smxfl[q] = s.sm_xw;
                pfl[q].push_back(s.pfl);
                pfl[q].back().gate = GATE_ENDING;
                gpfl[q].push_back(s.grid_pfl);
                if (s.sm_p > smpfl[q]) smpfl[q] = s.sm_p;
            }
            if (s.xw) {
                const int q = s.xw == 1 ? 0 : s.xw == 2 ? 1 : 2;
                xw[q].push_back(s.x);
                xw[q].back().gate = GATE_RUNNING;
                gxw[q].push_back(s.grid_xw);
                if (s.sm_xw > smxw[q]) smxw[q] = s.sm_xw;
            } else {
                x.push_back(s.x);
                x.back().gate = GATE_RUNNING;
                gx.push_back(s.grid_x);
                if (s.sm_x > smx) smx = s.sm_x;
            }
            if (s.epl) {
                const int q = s.epl == 1 ? 0 : s.epl == 2 ? 1 : 2;
                pa[q].push_back(s.pl);
                pa[q].back().gate = GATE_RUNNING;
                gf[q].push_back(s.grid_pf);
                gi[q].push_back(s.grid_pi);
                if (s.sm_p > smp[q]) smp[q] = s.sm_p;
                continue;
            }
            z.push_back(s.z); z.back().gate = GATE_RUNNING;
            yf.push_back(s.yf); yf.back().gate = GATE_RUNNING;
            yi.push_back(s.yi); yi.back().gate = GATE_RUNNING;
            gz.push_back(s.grid_z); gy.push_back(s.grid_y);
            if (s.sm_z > smz) smz = s.sm_z;
            if (s.sm_y > smy) smy = s.sm_y;
        }
        for (int q = 0; q < 3 && e == cudaSuccess; q++) {
            e = put_table(b, BL_PF1 + q, pa[q], gf[q], smp[q]);
            if (e == cudaSuccess) e = put_table(b, BL_PI1 + q, pa[q], gi[q], smp[q]);
        }
        if (e == cudaSuccess) e = put_table(b, BL_Z, z, gz, smz);
        if (e == cudaSuccess) e = put_table(b, BL_YF, yf, gy, smy);
        if (e == cudaSuccess) e = put_table(b, BL_YI, yi, gy, smy);
        if (e == cudaSuccess) e = put_table(b, BL_X, x, gx, smx);
        for (int q = 0; q < 3 && e == cudaSuccess; q++) e = put_table(b, BL_XW1 + q, xw[q], gxw[q], smxw[q]);
        for (int q = 0; q < 3 && e == cudaSuccess; q++) {
            e = put_table(b, BL_XFL1 + q, xfl[q], gxfl[q], smxfl[q]);
            if (e == cudaSuccess) e = put_table(b, BL_PFL1 + q, pfl[q], gpfl[q], smpfl[q]);
        }
    }
    {
        std::vector<NrArgs<T>> nr;
        std::vector<int> g;
        for (Ctx* c : b.slots) {
            nr.push_back(nrloop<T>(*c).a);
            nr.back().gate = GATE_RUNNING;
            g.push_back(nrloop<T>(*c).grid);
        }
        if (e == cudaSuccess) e = put_table(b, BL_NR, nr, g, 0);
    }
    if (sizeof(T) == 4) {
        std::vector<NrArgs<double>> nr;
        std::vector<FoldArgs> f;
        std::vector<int> g, gf;
        for (Ctx* c : b.slots) {
            nr.push_back(c->ks->nr64.a);
            nr.back().gate = GATE_ENDING;
            g.push_back(c->ks->nr64.grid);
            f.push_back(c->ks->fold);
            f.back().gate = GATE_ENDING;
            gf.push_back(c->ks->grid_fold);
        }
        if (e == cudaSuccess) e = put_table(b, BL_REFINE, nr, g, 0);
        if (e == cudaSuccess) e = put_table(b, BL_FOLD, f, gf, 0);
    }
    {
        std::vector<MacroArgs> m;
        // head and tail tables per arithmetic type: [0] FP64, [1] FP32 (FP32 bulk
        // without GND)
        std::vector<BeginArgs> bg[2];
        std::vector<EndArgs> en[2];
        std::vector<EndReduceArgs> er;
        std::vector<Macro*> mp;
        std::vector<int> gm, gb[2], ge[2], g1;
        for (Ctx* c : b.slots) {
            const int t = head_tail_fp32(*c) ? 1 : 0;
            m.push_back(c->ks->mac);
            gm.push_back(c->ks->mac.nblk);
            bg[t].push_back(c->ks->beg);
            bg[t].back().gate = GATE_BEGIN;
            gb[t].push_back(c->ks->grid_begin);
            en[t].push_back(c->ks->end);
            en[t].back().gate = GATE_ENDING;
            ge[t].push_back(c->ks->grid_end);
            er.push_back(c->ks->endr);
            er.back().gate = GATE_ENDING;
            g1.push_back(1);
            mp.push_back(c->macro);
        }
        if (e == cudaSuccess) e = put_table(b, BL_MACRO, m, gm, 0);
        if (e == cudaSuccess) e = put_table(b, BL_BEGIN, bg[0], gb[0], 0);
        if (e == cudaSuccess) e = put_table(b, BL_BEGIN32, bg[1], gb[1], 0);
        if (e == cudaSuccess) e = put_table(b, BL_END, en[0], ge[0], 0);
        if (e == cudaSuccess) e = put_table(b, BL_END32, en[1], ge[1], 0);
        if (e == cudaSuccess) e = put_table(b, BL_ENDR, er, g1, 0);
        if (e == cudaSuccess) e = put_table(b, BL_MBEGIN, mp, g1, 0);
        // BL_MBEGIN: nblk counts the slots
        b.L[BL_MBEGIN].nblk = (int)n;
    }
    return e;
}

static cudaError_t build_tables(Batch& b) {
    return b.precision == 0 ? build_tables_t<double>(b) : build_tables_t<float>(b);
}

// Record one round into b.graph (stream capture into the conditional body).
static int build_graph(Batch& b) {
    free_graph(b);
    const int n = (int)b.slots.size();
    const bool one = n == 1;
    Ctx* c0 = b.slots[0];
    Macro* const* dm = (Macro* const*)b.dtab[BL_MBEGIN];
    BCK(cudaGraphCreate(&b.graph, 0));
    cudaGraphConditionalHandle h;
    BCK(cudaGraphConditionalHandleCreate(&h, b.graph, 1, cudaGraphCondAssignDefault));
    // prologue, captured into the round graph itself (the kernel that sets the
    // WHILE condition belongs to the same graph as the handle)
    long long saved = one ? c0->launches : 0;
    BCK(cudaStreamBeginCaptureToGraph(b.stream, b.graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int np = 0;
    if (one) {
        cudaStream_t cs = c0->stream;
        c0->stream = b.stream;
        launch_macro_begin(*c0, GATE_BEGIN);
        launch_begin(*c0, GATE_BEGIN);
        c0->stream = cs;
        np = 2;
    } else {
        np = launch_begin_batch(b.L, b.stream);
    }
    k_round_start<<<1, ADVANCE_THREADS, 0, b.stream>>>(dm, n, b.dtk, b.dtk + 1, h);
    np++;
    // forward transforms of the round's first iteration (the body computes
    // those of the next iteration)
    if (one) {
        cudaStream_t cs = c0->stream;
        c0->stream = b.stream;
        launch_spectral(*c0, GATE_RUNNING, SPEC_FWD);
        c0->stream = cs;
        np += (c0->precision ? c0->ks->s32.epl : c0->ks->s64.epl) ? 2 : 3;
    } else {
        np += launch_spectral_batch(b.precision, b.L, b.stream, SPEC_FWD);
    }
    std::vector<cudaGraphNode_t> deps;
    {
        cudaStreamCaptureStatus cst;
        const cudaGraphNode_t* d = nullptr;
        size_t nd = 0;
        cudaError_t ce = cudaStreamGetCaptureInfo(b.stream, &cst, nullptr, nullptr, &d, nullptr, &nd);
        if (ce == cudaSuccess && d) deps.assign(d, d + nd);
        cudaGraph_t g_out = nullptr;
        cudaError_t ce2 = cudaStreamEndCapture(b.stream, &g_out);
        if (ce != cudaSuccess || ce2 != cudaSuccess || deps.empty())
            return bfail(EVPG_ERR_CUDA, "prologue capture: %s / %s", cudaGetErrorString(ce), cudaGetErrorString(ce2));
    }
    cudaGraphNode_t wn;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    BCK(cudaGraphAddNode(&wn, b.graph, deps.data(), nullptr, deps.size(), &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaGraphConditionalHandle hif;
    BCK(cudaGraphConditionalHandleCreate(&hif, b.graph, 0, cudaGraphCondAssignDefault));
    // body: the equilibrium iteration of every running RVE ...
    BCK(cudaStreamBeginCaptureToGraph(b.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    // inverse transforms (DisGrad update) and the NR sweep, then the macro
    // update on a side branch while the main branch computes the next
    // iteration's forward transforms: they read the new stress and write only
    // the spectrum buffer, and the macro update's results (loop test, mixed-BC
    // correction) are needed first by the next inverse transforms. Per RVE the
    // arithmetic is that of the launch-by-launch iteration.
    int nb = 0, nt = 0;
    cudaError_t fe = cudaSuccess;  // fork/join of the side branch
    if (one) {
        cudaStream_t cs = c0->stream;
        c0->stream = b.stream;
        launch_spectral(*c0, GATE_RUNNING, SPEC_INV);
        launch_nr(*c0, 0, GATE_RUNNING);
        fe = cudaEventRecord(b.ev_fork, b.stream);
        if (fe == cudaSuccess) fe = cudaStreamWaitEvent(b.side, b.ev_fork, 0);
        if (fe == cudaSuccess) {
            c0->stream = b.side;
            launch_macro(*c0);
            fe = cudaEventRecord(b.ev_join, b.side);
            c0->stream = b.stream;
        }
        launch_spectral(*c0, GATE_RUNNING, SPEC_FWD);
        if (fe == cudaSuccess) fe = cudaStreamWaitEvent(b.stream, b.ev_join, 0);
        const int fused = c0->precision ? c0->ks->s32.epl : c0->ks->s64.epl;
        nb = (fused ? 3 : 5) + 2;
        c0->stream = cs;
    } else {
        nb = launch_spectral_batch(b.precision, b.L, b.stream, SPEC_INV) + 2;
        launch_nr_batch(b.precision, b.nr_mode, b.L[BL_NR], b.stream);
        fe = cudaEventRecord(b.ev_fork, b.stream);
        if (fe == cudaSuccess) fe = cudaStreamWaitEvent(b.side, b.ev_fork, 0);
        if (fe == cudaSuccess) {
            launch_macro_batch(b.L[BL_MACRO], b.side);
            fe = cudaEventRecord(b.ev_join, b.side);
        }
        nb += launch_spectral_batch(b.precision, b.L, b.stream, SPEC_FWD);
        if (fe == cudaSuccess) fe = cudaStreamWaitEvent(b.stream, b.ev_join, 0);
    }
    if (fe != cudaSuccess) {
        cudaGraph_t g_out = nullptr;
        cudaStreamEndCapture(b.stream, &g_out);
        if (one) c0->launches = saved;
        return bfail(EVPG_ERR_CUDA, "body fork/join: %s", cudaGetErrorString(fe));
    }
    k_if_ending<<<1, ADVANCE_THREADS, 0, b.stream>>>(dm, n, b.dtk, hif);
    nb++;
    std::vector<cudaGraphNode_t> bdeps;
    {
        cudaStreamCaptureStatus cst;
        const cudaGraphNode_t* d = nullptr;
        size_t nd = 0;
        cudaError_t ce = cudaStreamGetCaptureInfo(b.stream, &cst, nullptr, nullptr, &d, nullptr, &nd);
        if (ce == cudaSuccess && d) bdeps.assign(d, d + nd);
        cudaGraph_t g_out = nullptr;
        cudaError_t ce2 = cudaStreamEndCapture(b.stream, &g_out);
        if (ce != cudaSuccess || ce2 != cudaSuccess || bdeps.empty()) {
            if (one) c0->launches = saved;
            return bfail(EVPG_ERR_CUDA, "body capture: %s / %s", cudaGetErrorString(ce), cudaGetErrorString(ce2));
        }
    }
    // ... then, only in iterations where some RVE's loop ended, its tail
    // (each kernel still gated per RVE) ...
    cudaGraphNode_t ifn;
    cudaGraphNodeParams ip = {cudaGraphNodeTypeConditional};
    ip.conditional.handle = hif;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    BCK(cudaGraphAddNode(&ifn, body, bdeps.data(), nullptr, bdeps.size(), &ip));
    BCK(cudaStreamBeginCaptureToGraph(b.stream, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal));
    if (one) {
        cudaStream_t cs = c0->stream;
        c0->stream = b.stream;
        if (c0->precision != 0) {
            launch_fold(*c0, GATE_ENDING);
            launch_nr(*c0, 1, GATE_ENDING);
            nt += 2 + spectral_flush_kernels(*c0);
        }
        launch_end(*c0, GATE_ENDING);
        nt += 2;
        c0->stream = cs;
    } else {
        nt += launch_end_batch(b.precision, b.nr_mode, b.L, b.stream);
    }
    {
        cudaGraph_t g_out = nullptr;
        cudaError_t ce = cudaStreamEndCapture(b.stream, &g_out);
        if (ce != cudaSuccess) {
            if (one) c0->launches = saved;
            return bfail(EVPG_ERR_CUDA, "tail capture: %s", cudaGetErrorString(ce));
        }
    }
    // ... and the loop control
    BCK(cudaStreamBeginCaptureToGraph(b.stream, body, &ifn, nullptr, 1, cudaStreamCaptureModeThreadLocal));
    k_advance<<<1, ADVANCE_THREADS, 0, b.stream>>>(dm, n, b.dtk, b.dtk + 1, h);
    nb++;
    cudaGraph_t body_out = nullptr;
    cudaError_t ce = cudaStreamEndCapture(b.stream, &body_out);
    if (one) c0->launches = saved;
    if (ce != cudaSuccess) return bfail(EVPG_ERR_CUDA, "body capture: %s", cudaGetErrorString(ce));
    BCK(cudaGraphInstantiate(&b.exec, b.graph, 0));
    b.prologue_kernels = np;
    b.body_kernels = nb;
    b.tail_kernels = nt;
    return EVPG_OK;
}

static int rebuild(Batch& b) {
    if (b.slots.empty()) return EVPG_OK;
    BCK(cudaStreamSynchronize(b.stream));
    free_graph(b);
    free_tables(b);
    BCK(build_tables(b));
    const int st = build_graph(b);
    if (st) return st;
    b.versions.clear();
    for (Ctx* c : b.slots) b.versions.push_back(c->version);
    b.dirty = false;
    return EVPG_OK;
}

static int set_slots(Batch& b, Ctx* const* ctxs, int n) {
    for (int i = 0; i < n; i++) {
        if (!ctxs[i]) return bfail(EVPG_ERR_ARG, "slot %d: null context", i);
        if (ctxs[i]->precision != b.precision || ctxs[i]->nr_mode != b.nr_mode)
            return bfail(EVPG_ERR_ARG, "slot %d: precision/NR mode differ from the batch", i);
        for (int j = 0; j < i; j++)
            if (ctxs[j] == ctxs[i]) return bfail(EVPG_ERR_ARG, "context in two slots");
        BCK(cudaStreamSynchronize(ctxs[i]->stream));
    }
    BCK(cudaStreamSynchronize(b.stream));
    b.slots.assign(ctxs, ctxs + n);
    if (n > b.cap) {
        if (b.hctl) cudaFreeHost(b.hctl);
        b.hctl = nullptr;
        BCK(cudaMallocHost((void**)&b.hctl, sizeof(IncrCtl) * (size_t)n));
        b.cap = n;
    }
    b.staged.assign((size_t)n, 0);
    b.dirty = true;
    return EVPG_OK;
}

// Stage slot i's next increment (copied to the device when the round starts).
static void stage(Batch& b, int i, const double udot_dt[3][3], int creep, const double dgavg[3][3],
                  double time_tot, double e_vm, int tail) {
    Ctx* c = b.slots[i];
    IncrCtl& k = b.hctl[i];
    double g9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    sym_to_b6<double>(udot_dt, k.udot9);
    k.udot9[6] = 0.5 * (udot_dt[0][1] - udot_dt[1][0]);
    k.udot9[7] = 0.5 * (udot_dt[0][2] - udot_dt[2][0]);
    k.udot9[8] = 0.5 * (udot_dt[1][2] - udot_dt[2][1]);
    if (creep && dgavg) {
        sym_to_b6<double>(dgavg, g9);
        g9[6] = 0.5 * (dgavg[0][1] - dgavg[1][0]);
        g9[7] = 0.5 * (dgavg[0][2] - dgavg[2][0]);
        g9[8] = 0.5 * (dgavg[1][2] - dgavg[2][1]);
    }
    memcpy(k.dgavg9, g9, sizeof g9);
    // DeltaTau_DRX*exp((t_last-TimeTot)/TimeStep/tau_DRX), t_last = -1E3*tau_DRX*TimeStep
    const double dt = c->m64.dt;
    const double t_last = -1E3 * c->tau_drx * dt;
    k.drx = c->delta_tau_drx * exp((t_last - time_tot) / dt / c->tau_drx);
    k.e_vm = e_vm;
    k.err0 = 2. * c->cfg.err_tol;
    k.creep = creep ? 1 : 0;
    k.tail = tail & (EVPG_TAIL_REORIENT | EVPG_TAIL_GND_GRADIENT);
    k.phase = PH_BEGIN;
    k.pad = 0;
    b.staged[i] = 1;
}

static int run_round(Batch& b, int kmax, int* ticks) {
    if (b.slots.empty()) return bfail(EVPG_ERR_ARG, "empty batch");
    bool changed = b.dirty;
    for (size_t i = 0; i < b.slots.size() && !changed; i++) changed = b.versions[i] != b.slots[i]->version;
    if (changed) {
        const int st = rebuild(b);
        if (st) return st;
    }
    for (size_t i = 0; i < b.slots.size(); i++)
        if (b.staged[i]) {
            BCK(cudaMemcpyAsync(b.slots[i]->macro, &b.hctl[i], sizeof(IncrCtl), cudaMemcpyHostToDevice, b.stream));
            b.staged[i] = 0;
        }
    b.htk[1] = kmax;
    BCK(cudaMemcpyAsync(b.dtk + 1, b.htk + 1, sizeof(int), cudaMemcpyHostToDevice, b.stream));
    BCK(cudaGraphLaunch(b.exec, b.stream));
    for (Ctx* c : b.slots)
        BCK(cudaMemcpyAsync(c->macro_host, c->macro, sizeof(Macro), cudaMemcpyDeviceToHost, b.stream));
    BCK(cudaMemcpyAsync(b.htk, b.dtk, 3 * sizeof(int), cudaMemcpyDeviceToHost, b.stream));
    BCK(cudaStreamSynchronize(b.stream));
    const int t = b.htk[0];
    const long long nl = b.prologue_kernels + (long long)t * b.body_kernels + (long long)b.htk[2] * b.tail_kernels;
    b.launches += nl;
    if (b.slots.size() == 1) b.slots[0]->launches += nl;
    b.rounds++;
    if (ticks) *ticks = t;
    return EVPG_OK;
}

static void destroy_batch(Batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    free_graph(*b);
    free_tables(*b);
    if (b->dtk) cudaFree(b->dtk);
    if (b->htk) cudaFreeHost(b->htk);
    if (b->hctl) cudaFreeHost(b->hctl);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    delete b;
}

static int create_batch(int precision, int nr_mode, cudaStream_t stream, Batch** out) {
    Batch* b = new Batch();
    b->precision = precision;
    b->nr_mode = nr_mode;
    cudaError_t e = cudaSuccess;
    if (stream) {
        b->stream = stream;
    } else {
        e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        b->own_stream = e == cudaSuccess;
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->dtk, 3 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(b->dtk, 0, 3 * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->htk, 3 * sizeof(int));
    if (e != cudaSuccess) {
        destroy_batch(b);
        return bfail(EVPG_ERR_CUDA, "batch creation: %s", cudaGetErrorString(e));
    }
    b->htk[0] = b->htk[1] = b->htk[2] = 0;
    *out = b;
    return EVPG_OK;
}

// Per-context batch of one used by evpg_increment (the context's own stream).
void free_solo(Ctx& c) {
    destroy_batch((Batch*)c.solo);
    c.solo = nullptr;
}

static void fill_iter(const Macro& m, evpg_iter_out* o) {
    o->err_e = m.err_e;
    o->err_s = m.err_s;
    o->err_e_sum = m.err_e_sum;
    o->err_s_sum = m.err_s_sum;
    memcpy(o->sig_avg, m.sig_avg, sizeof o->sig_avg);
    memcpy(o->sig_avg_ph1, m.sig_avg1, sizeof o->sig_avg_ph1);
    memcpy(o->ddisgrad, m.dE, sizeof o->ddisgrad);
    memcpy(o->ddisgrad_acum, m.dE_acum, sizeof o->ddisgrad_acum);
    o->s_vm = m.s_vm;
    o->s_vm1 = m.s_vm1;
    o->iter = m.iter;
    o->converged = m.converged;
}

static void fill_incr(const Macro& m, evpg_incr_out* o) {
    double e6[6], d6[6];
    memcpy(e6, m.eps_avg6, sizeof e6);
    memcpy(d6, m.edot_avg6, sizeof d6);
    b6_to_sym<double>(e6, o->eps_avg);
    b6_to_sym<double>(d6, o->edot_avg);
    memcpy(o->rho_avg, m.rho_avg, sizeof o->rho_avg);
    o->nr_iterations = m.nr_iters;
}

}  // namespace evpg

using namespace evpg;

extern "C" {

const char* evpg_batch_last_error(void) { return evpg_last_error(); }

int evpg_batch_create(int32_t precision, int32_t nr_mode, void** out) {
    if (!out) return bfail(EVPG_ERR_ARG, "null argument");
    *out = nullptr;
    if (precision != EVPG_FP64 && precision != EVPG_FP32_BULK) return bfail(EVPG_ERR_ARG, "precision");
    if (nr_mode != EVPG_NR_PLAIN && nr_mode != EVPG_NR_LINESEARCH) return bfail(EVPG_ERR_ARG, "nr_mode");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return bfail(EVPG_ERR_NO_DEVICE, "no CUDA device");
    Batch* b = nullptr;
    const int st = create_batch(precision, nr_mode, nullptr, &b);
    if (st) return st;
    *out = b;
    return EVPG_OK;
}

int evpg_batch_destroy(void* batch) {
    destroy_batch((Batch*)batch);
    return EVPG_OK;
}

int evpg_batch_set(void* batch, void* const* ctxs, int32_t n) {
    Batch* b = (Batch*)batch;
    if (!b || (n > 0 && !ctxs) || n < 0) return bfail(EVPG_ERR_ARG, "bad argument");
    return set_slots(*b, (Ctx* const*)ctxs, n);
}

int evpg_batch_stage(void* batch, int32_t slot, const double udot_dt[3][3], int32_t creep,
                     const double disgrad_avg_actual[3][3], double time_tot, double e_vm, int32_t tail) {
    Batch* b = (Batch*)batch;
    if (!b || !udot_dt || slot < 0 || slot >= (int)b->slots.size()) return bfail(EVPG_ERR_ARG, "bad argument");
    if (creep && !disgrad_avg_actual) return bfail(EVPG_ERR_ARG, "creep needs disgrad_avg_actual");
    stage(*b, slot, udot_dt, creep, disgrad_avg_actual, time_tot, e_vm, tail);
    return EVPG_OK;
}

int evpg_batch_round(void* batch, int32_t max_ticks, int32_t* ticks) {
    Batch* b = (Batch*)batch;
    if (!b || max_ticks < 1) return bfail(EVPG_ERR_ARG, "bad argument");
    return run_round(*b, max_ticks, ticks);
}

int evpg_batch_slot(void* batch, int32_t slot, int32_t* phase, int32_t* status, evpg_iter_out* it,
                    evpg_incr_out* inc) {
    Batch* b = (Batch*)batch;
    if (!b || slot < 0 || slot >= (int)b->slots.size()) return bfail(EVPG_ERR_ARG, "bad argument");
    const Macro& m = *b->slots[slot]->macro_host;
    if (phase) *phase = m.ctl.phase;
    if (status) *status = m.status;
    if (it) fill_iter(m, it);
    if (inc) fill_incr(m, inc);
    return EVPG_OK;
}

int evpg_batch_launch_count(void* batch, int64_t* n) {
    Batch* b = (Batch*)batch;
    if (!b || !n) return bfail(EVPG_ERR_ARG, "bad argument");
    *n = b->launches;
    return EVPG_OK;
}

int evpg_increment(void* ctx, const double udot_dt[3][3], int32_t creep, const double disgrad_avg_actual[3][3],
                   double time_tot, double e_vm, int32_t tail, evpg_iter_out* it, evpg_incr_out* inc) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !udot_dt) return bfail(EVPG_ERR_ARG, "null argument");
    if (creep && !disgrad_avg_actual) return bfail(EVPG_ERR_ARG, "creep needs disgrad_avg_actual");
    if (c->prof.on) {
        // per-kernel timing needs the launch-by-launch path
        int st = evpg_increment_begin(ctx, udot_dt, creep, disgrad_avg_actual, time_tot);
        if (!st) st = evpg_equilibrium_solve(ctx, e_vm, it);
        if (!st) st = evpg_increment_end(ctx, tail, inc);
        return st;
    }
    Batch* b = (Batch*)c->solo;
    if (!b || b->stream != c->stream) {
        free_solo(*c);
        int st = create_batch(c->precision, c->nr_mode, c->stream, &b);
        if (st) return st;
        c->solo = b;
        st = set_slots(*b, &c, 1);
        if (st) return st;
    }
    stage(*b, 0, udot_dt, creep, disgrad_avg_actual, time_tot, e_vm, tail);
    int ticks = 0;
    const int st = run_round(*b, c->cfg.iter_max + 1, &ticks);
    if (st) return st;
    const Macro& m = *c->macro_host;
    if (it) fill_iter(m, it);
    if (inc) fill_incr(m, inc);
    if (m.status) return bfail(m.status, "%s", evpg_status_string(m.status));
    if (m.ctl.phase != PH_ENDED) return bfail(EVPG_ERR_CUDA, "increment did not finish (%d ticks)", ticks);
    return EVPG_OK;
}

}  // extern "C"
