#!/usr/bin/env python
"""Benchmark of the EVP-FFT equilibrium iteration on one GB300 per rank.

Workload (the precision-form configuration): a 128^3 RVE of FCC Cu with 1000
seeded periodic Voronoi grains, uniform-random orientations, initial SSD
density log-uniform in [5e11, 5e12] m^-2 per grain, uniaxial z tension at
1e-3/s with stress-free lateral faces, 2e-4 strain per increment (5% in 250
increments), Err 1e-5. The NR uses the reference's line search
(NR_MODIFIED): with the plain update the reference itself aborts on this
material at the second increment.

One step = one increment (increment head, the whole equilibrium loop and the
increment tail). W warm-up increments run first; K increments are timed with
CUDA events on the context's stream. metric = voxel-iterations/s =
sum over timed increments of N x equilibrium iterations / time.

The headline is the FP32-bulk form; the plain FP64 form is timed on the same
increments of its own run for the speed-up and error figures.

  python bench.py [--steps K] [--warmup W] [--impl gpu|reference] [--grid 128]
                  [--grains 1000] [--fp64-steps K64] [--forms batch,serve]
  python bench.py --series 25     per-increment FP32-bulk vs FP64 errors (untimed)

Under torchrun each rank runs an independent replica (the path does not
shard: one RVE per GPU); value = all ranks' voxel-iterations / max time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel-iters/s 128^3 FP32-bulk vs FP64 (<=1e-4 sigma err)"
# dram__bytes_read.sum + dram__bytes_write.sum of one FP32 NR sweep per voxel, from an
# ncu capture of the 96^3 / 422-grain case (traffic grows with N: every voxel's state is
# read and written once); scaled by N for the roofline's "traffic".
NR_DRAM_BYTES_PER_VOXEL = 487.8
# values of P bytes the per-voxel constitutive update must move (strain, plastic strain,
# lambda, rho_s, rho_m, orientation in; sigma, rho_m out)
NR_ALG_VALUES_PER_VOXEL = 69
# FP32 operations (2 per FFMA, 1 per FADD/FMUL) per Newton step of the FP32 NR sweep,
# from the thread-level instruction counters of an ncu capture of every NR sweep of one
# increment of the 96^3 / 422-grain RVE (2267 per voxel-sweep at 1.956 Newton steps)
NR_FP32_FLOP_PER_NEWTON_STEP = 1158.7
# 152 SMs x 128 FP32 lanes x 2 FLOP x 2.07 GHz (maximum SM clock)
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
FP32_PEAK_SOURCE = "derived: 152 SMs x 128 FP32 lanes x 2 FLOP/FFMA x 2070 MHz"
UNIT = "voxel-iterations/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    p.add_argument("--grid", type=int, default=128, help="RVE edge length in voxels")
    p.add_argument("--grains", type=int, default=1000)
    p.add_argument("--fp64-steps", type=int, default=None,
                   help="FP64 increments timed (default: the same increments as the FP32-bulk form)")
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--workdir", default=None)
    p.add_argument("--batch-count", type=int, default=64)
    p.add_argument("--batch-steps", type=int, default=10)
    p.add_argument("--batch-steps-fp64", type=int, default=3)
    p.add_argument("--serve-requests", type=int, default=24)
    p.add_argument("--serve-rates", default="0.5,2,16")
    p.add_argument("--serve-fp64-requests", type=int, default=8,
                   help="requests of the FP32-bulk vs FP64 serving comparison (same stream, both forms)")
    p.add_argument("--serve-fp64-rate", type=float, default=0.25)
    p.add_argument("--series", type=int, default=0,
                   help="precision series only: run this many increments of both forms and print the "
                        "per-increment macro stress and field L2 errors of FP32-bulk against FP64")
    p.add_argument("--forms", default="batch,serve", help="extra forms to measure ('' for none)")
    p.add_argument("--no-tune", action="store_true",
                   help="keep the default spectral schedule (no autotuner trials; for launch-list profiling, "
                        "where the trial timings are not the kernels' own)")
    return p.parse_args()


def workload_config(a):
    return {"workload": "%d^3 RVE, %d Voronoi grains, FCC Cu, rho0 log-uniform [5e11,5e12]/grain, "
                        "z tension 1e-3/s, 2e-4/increment, line-search NR" % (a.grid, a.grains),
            "grid": [a.grid, a.grid, a.grid], "grains": a.grains, "increments_per_step": 1,
            "err_tol": 1e-5, "seed": 2025,
            "l2": "inputs larger than L2 (per-voxel state ~2.5 KB/voxel, GBs resident)"}


def make_workload(a, d):
    from srx_gb300 import rve
    job = rve.Job(n=(a.grid,) * 3, load="tension", rate=1e-3, strain_per_step=2e-4, n_steps=250,
                  err=1e-5, iter_max=1000)
    return rve.make_case(d, (a.grid,) * 3, a.grains, 2025, job, rho0=(0.5, 5.0))


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                sm.append(float(f[1]))
                mx.append(float(f[2]))
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        except (OSError, ValueError):
            pass
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce(x, op):
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def allmax(ws, x):
    if ws == 1:
        return x
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.MAX)


def allsum(ws, x):
    if ws == 1:
        return x
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.SUM)


# ------------------------------------------------------------- CPU oracle

def oracle_lib():
    so = os.path.join(ROOT, "oracle", "_build", "libevporacle.so")
    if not os.path.exists(so):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    L = C.CDLL(so)
    L.evo_open.restype = C.c_void_p
    L.evo_open.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]
    L.evo_close.argtypes = [C.c_void_p]
    L.evo_set_nr_mode.argtypes = [C.c_void_p, C.c_int]
    L.evo_set_threads.argtypes = [C.c_int]
    L.evo_begin.argtypes = [C.c_void_p]
    L.evo_iteration.argtypes = [C.c_void_p]
    return L


def cpu_sample(case, iters, threads):
    """The oracle (CPU restatement of the reference, line-search NR) on the
    same RVE: increment head, then `iters` equilibrium iterations, timed."""
    L = oracle_lib()
    L.evo_set_threads(threads)
    err = C.create_string_buffer(512)
    h = L.evo_open(case["input"].encode(), case["rho0"].encode(), err, 512)
    if not h:
        raise RuntimeError(err.value.decode())
    L.evo_set_nr_mode(h, 1)
    L.evo_begin(h)
    times = []
    for _ in range(iters):
        t = time.perf_counter()
        st = L.evo_iteration(h)
        times.append(time.perf_counter() - t)
        if st:
            raise RuntimeError("oracle iteration status %d" % st)
    L.evo_close(h)
    return times


# ------------------------------------------------------------------ arms

def reference_arm(a, ws, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory(dir=a.workdir) as d:
        case = make_workload(a, d)
        times = cpu_sample(case, a.warmup + a.steps, threads)
    N = a.grid ** 3
    t = sum(times[a.warmup:])
    value = N * a.steps / t
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * t / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(a),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "one step = one equilibrium iteration (FFT, Green, inverse FFT, "
                                   "line-search NR, get_smacro) of increment 0 of the %d^3 RVE; "
                                   "FFT is the project's CPU mixed-radix DFT, not FFTW" % a.grid},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def batch_leg(a, evpg, root):
    """Batching form: RVEs of uneven grids, loads and rates advanced in one
    batch (one launch per kernel over all RVEs, one CUDA graph per round),
    against the same RVEs run one after another alone (their own per-increment
    graphs). Host wall time around synchronous calls. FP32-bulk runs
    --batch-steps increments per RVE, FP64 --batch-steps-fp64."""
    from srx_gb300 import workloads
    out = {"rves": a.batch_count}
    for prec, tag, steps in ((evpg.FP32_BULK, "fp32", a.batch_steps), (evpg.FP64, "fp64", a.batch_steps_fp64)):
        cases = workloads.batch_set(os.path.join(root, "batch_" + tag), count=a.batch_count, steps=steps)
        if tag == "fp32":
            out.update({"grids": sorted(set(c["n"] for c in cases)), "voxels": int(sum(c["N"] for c in cases)),
                        "loads": {k: sum(1 for c in cases if c["load"] == k)
                                  for k in ("tension", "compression", "shear")}})
        nsteps = [steps] * len(cases)
        jobs = [evpg.Job(c["input"], c["rho0"], precision=prec, nr_mode=evpg.NR_LINESEARCH) for c in cases]
        for j in jobs:
            if not a.no_tune:
                j.tune()  # searched once per grid, cached for the others
        t0 = time.perf_counter()
        its, rounds = evpg.run_batched(jobs, nsteps, max_ticks=32)
        tb = time.perf_counter() - t0
        vi = float(sum(c["N"] * sum(i) for c, i in zip(cases, its)))
        for j in jobs:
            j.close()
        rec = {"value": vi / tb, "unit": UNIT, "increments_per_rve": steps, "seconds": tb, "rounds": rounds,
               "iterations": int(sum(sum(i) for i in its))}
        if tag == "fp32":
            jobs = [evpg.Job(c["input"], c["rho0"], precision=prec, nr_mode=evpg.NR_LINESEARCH) for c in cases]
            for j in jobs:
                if not a.no_tune:
                    j.tune()
            t0 = time.perf_counter()
            its_alone = [[j.increment(k) for k in range(steps)] for j in jobs]
            ta = time.perf_counter() - t0
            for j in jobs:
                j.close()
            rec["alone_sequential"] = {"value": vi / ta, "seconds": ta,
                                       "same_iterations": its_alone == its}
            rec["batch_over_alone"] = ta / tb
        out[tag] = rec
    out["round_tick"] = batch_tick_cost(a, evpg, root)
    return out


def batch_tick_cost(a, evpg, root):
    """Per-iteration cost of a round graph when the RVEs are tiny: 64 copies
    of one 8^3 RVE (all converge in the same iteration), so the wall time per
    equilibrium iteration is the cost of one pass of the round graph's body
    (its kernel nodes with almost no voxels, the conditional node, the
    launch gaps)."""
    from srx_gb300 import rve
    c = rve.make_case(os.path.join(root, "tick8"), (8, 8, 8), 4, 11,
                      rve.Job(n=(8, 8, 8), load="tension", n_steps=4))
    res = {}
    for prec, tag in ((evpg.FP32_BULK, "fp32"), (evpg.FP64, "fp64")):
        jobs = [evpg.Job(c["input"], None, precision=prec, nr_mode=evpg.NR_LINESEARCH) for _ in range(64)]
        evpg.run_batched(jobs, [1] * 64, max_ticks=32)  # warm-up increment, graph capture
        t0 = time.perf_counter()
        its, rounds = evpg.run_batched(jobs, [3] * 64, max_ticks=32)
        t = time.perf_counter() - t0
        for j in jobs:
            j.close()
        ticks = sum(its[0])
        res[tag] = {"us_per_iteration": 1e6 * t / ticks, "iterations": ticks, "rounds": rounds,
                    "rves": 64, "grid": [8, 8, 8]}
    return res


def serve_run(evpg, base, rate, prec, budget):
    with evpg.Server(precision=prec, nr_mode=evpg.NR_LINESEARCH, hbm_budget=budget,
                     max_slots=64, round_ticks=16, loaders=4) as srv:
        t0 = time.perf_counter()
        for c in base:
            dt = t0 + c["t"] / rate - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            srv.submit(c["input"], c["steps"], rho0=c["rho0"], switch_step=c["switch"],
                       switch_input=c["switch_input"])
        srv.wait(1800)
        st = srv.stats()
    return {"solves_per_s": st.solves_per_s, "solve_p50_s": st.solve_p50, "solve_p99_s": st.solve_p99,
            "increment_p50_s": st.incr_p50, "increment_p99_s": st.incr_p99,
            "completed": st.completed, "failed": st.failed, "rounds": st.rounds,
            "iterations": int(st.iterations), "span_s": st.span}


def serve_leg(a, evpg, root, budget):
    """Serving form: Poisson request streams through the continuous-batching
    server; latency per solve and per increment, solves/s. FP32-bulk at the
    --serve-rates (the lowest leaves the GPU mostly idle between requests:
    unloaded latency), then one shorter stream served by both forms."""
    from srx_gb300 import workloads
    rates = [float(r) for r in a.serve_rates.split(",") if r]
    base = workloads.serve_stream(os.path.join(root, "serve"), count=a.serve_requests, rate_hz=1.0,
                                  steps=(2, 4), distinct=min(12, a.serve_requests))
    out = {"requests": len(base), "grids": sorted(set(c["n"] for c in base)),
           "increments_per_request": [2, 4], "rates": {}}
    for rate in rates:
        out["rates"][str(rate)] = serve_run(evpg, base, rate, evpg.FP32_BULK, budget)
    if a.serve_fp64_requests > 0:
        short = base[:a.serve_fp64_requests]
        cmp = {"requests": len(short), "rate": a.serve_fp64_rate}
        for prec, tag in ((evpg.FP32_BULK, "fp32"), (evpg.FP64, "fp64")):
            cmp[tag] = serve_run(evpg, short, a.serve_fp64_rate, prec, budget)
        out["fp32_vs_fp64"] = cmp
    return out


def gpu_arm(a, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    from srx_gb300 import build
    build.build()
    from srx_gb300 import evpg
    L = evpg.lib()
    L.evpg_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    L.evpg_profile.argtypes = [C.c_void_p, C.c_int32]
    L.evpg_profile_read.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_int32]
    L.evpg_launch_count.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    N = a.grid ** 3

    with tempfile.TemporaryDirectory(dir=a.workdir) as d:
        case = make_workload(a, d)
        stream = torch.cuda.Stream()

        def open_job(prec):
            j = evpg.Job(case["input"], case["rho0"], precision=prec, nr_mode=evpg.NR_LINESEARCH)
            evpg.check(L.evpg_set_stream(j.ctx, C.c_void_p(stream.cuda_stream)))
            return j

        def launches(j):
            n = C.c_int64()
            evpg.check(L.evpg_launch_count(j.ctx, C.byref(n)))
            return n.value

        # ---------------- FP32 bulk: headline
        j32 = open_job(evpg.FP32_BULK)
        tune32 = {"gain": None if a.no_tune else j32.tune(), "schedule": j32.schedule(),
                  "variant": list(j32.variant())}
        for s in range(a.warmup):
            j32.increment(s)
        barrier(ws)
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps + 1)]
        iters32, sig32, svm32 = [], [], []
        l0 = launches(j32)
        with Clocks(local) as clk:
            ev[0].record(stream)
            for k, s in enumerate(range(a.warmup, a.warmup + a.steps)):
                iters32.append(j32.increment(s))
                sc = j32.scalars()
                sig32.append(sc[7:16].copy())
                svm32.append(float(sc[5]))
                ev[k + 1].record(stream)
            torch.cuda.synchronize()
        nlaunch = launches(j32) - l0
        inc32 = [ev[k].elapsed_time(ev[k + 1]) for k in range(a.steps)]
        t32 = ev[0].elapsed_time(ev[a.steps]) / 1e3
        clocks = clk.summary()
        barrier(ws)
        tmax = allmax(ws, t32)
        vi = allsum(ws, float(N * sum(iters32)))
        value = vi / tmax
        # fields after the last timed increment (outside the timed region)
        f32 = {"sig": j32.download(evpg.F_SIG6), "rho_s": j32.download(evpg.F_RHO_S)}

        # ---------------- e2e through the C ABI with host buffers
        pin = torch.empty(N * 6, dtype=torch.float64, pin_memory=True)
        hostv = pin.numpy().reshape(N, 6)
        e2e_iters = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s0 = a.warmup + a.steps
        for s in range(s0, s0 + a.e2e_steps):
            e2e_iters += j32.increment(s)  # the increment's controls (184 B) go down by one copy
            j32.download_into(evpg.F_SIG6, hostv)  # pinned: packed on the device, one D2H per chunk
        torch.cuda.synchronize()
        te2e = time.perf_counter() - t0
        e2e_value = allsum(ws, float(N * e2e_iters)) / allmax(ws, te2e)

        # ---------------- per-kernel times (profiling run, one increment)
        names = ["fwd_z", "fwd_y", "x_green", "inv_y", "inv_z", "nr", "macro", "begin", "end",
                 "refine"]
        ms = (C.c_double * 10)()
        nl = (C.c_int64 * 10)()

        def profile_increment(j, s):
            evpg.check(L.evpg_profile(j.ctx, 1))
            it = j.increment(s)
            newton = float(j.scalars()[33])
            evpg.check(L.evpg_profile_read(j.ctx, ms, nl, 10))
            evpg.check(L.evpg_profile(j.ctx, 0))
            pr = {nm: {"ms_total": ms[i], "launches": int(nl[i]),
                       "ms_per_launch": ms[i] / nl[i] if nl[i] else None} for i, nm in enumerate(names)}
            return pr, it, newton

        prof, it_prof, newton_prof = profile_increment(j32, s0 + a.e2e_steps)
        j32.close()

        # ---------------- FP64 plain form on the same increments
        k64 = a.steps if a.fp64_steps is None else max(1, min(a.fp64_steps, a.steps))
        j64 = open_job(evpg.FP64)
        tune64 = {"gain": None if a.no_tune else j64.tune(), "schedule": j64.schedule()}
        for s in range(a.warmup):
            j64.increment(s)
        torch.cuda.synchronize()
        e64 = [torch.cuda.Event(enable_timing=True) for _ in range(k64 + 1)]
        iters64, sig64, svm64 = [], [], []
        e64[0].record(stream)
        for k, s in enumerate(range(a.warmup, a.warmup + k64)):
            iters64.append(j64.increment(s))
            sc = j64.scalars()
            sig64.append(sc[7:16].copy())
            svm64.append(float(sc[5]))
            e64[k + 1].record(stream)
        torch.cuda.synchronize()
        inc64 = [e64[k].elapsed_time(e64[k + 1]) for k in range(k64)]
        t64 = e64[0].elapsed_time(e64[k64]) / 1e3
        f64 = {"sig": j64.download(evpg.F_SIG6), "rho_s": j64.download(evpg.F_RHO_S)} if k64 == a.steps else None
        # per-kernel times of one FP64 increment (launch by launch)
        prof64, it64p, _ = profile_increment(j64, a.warmup + k64)
        prof64 = {k: v for k, v in prof64.items() if v["launches"]}
        prof64["iterations"] = it64p
        j64.close()

        forms = {}
        wanted = [f for f in a.forms.split(",") if f]
        if "batch" in wanted:
            forms["batching"] = batch_leg(a, evpg, d)
        if "serve" in wanted:
            free, _ = torch.cuda.mem_get_info()
            forms["serving"] = serve_leg(a, evpg, d, int(0.8 * free))

    value64 = N * sum(iters64) / t64
    ms_inc32 = 1e3 * t32 / a.steps
    ms_inc64 = 1e3 * t64 / k64
    macro_err = [float(np.max(np.abs(sig32[i] - sig64[i])) / np.max(np.abs(sig64[i]))) for i in range(k64)]
    l2 = (lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y)))
    field_err = ({k: l2(f32[k], f64[k]) for k in ("sig", "rho_s")} if f64 is not None else None)
    precision = {
        "increments": list(range(a.warmup, a.warmup + k64)),
        "fp32_ms_per_increment": inc32[:k64], "fp64_ms_per_increment": inc64,
        "fp32_over_fp64_per_increment": (sum(inc64) / k64) / (sum(inc32[:k64]) / k64),
        "fp32_over_fp64_per_voxel_iteration": (N * sum(iters32[:k64]) / (sum(inc32[:k64]) / 1e3)) / value64,
        "same_iterations": iters32[:k64] == iters64,
        "fp32_macro_sigma_rel_err": macro_err,
        "fp32_svm_rel_err": [abs(svm32[i] - svm64[i]) / abs(svm64[i]) for i in range(k64)],
        "fp32_field_l2_err": field_err,
        "field_l2_at_increment": a.warmup + a.steps - 1 if field_err else None,
        "bounds": {"macro_sigma": 1e-4, "field_l2": 1e-3},
    }

    # roofline of the dominant kernel group (by time in the profiling run)
    dom = max(("fwd_z", "fwd_y", "x_green", "inv_y", "inv_z", "nr"), key=lambda k: prof[k]["ms_total"])
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    hbm_src = "measured" if "hbm_gbs" in peaks else "fallback"
    Nh = a.grid * a.grid * (a.grid // 2 + 1)
    P = 4  # FP32 bulk
    # Algorithmic HBM bytes per launch. Spectral passes: the half spectra
    # they must read and write between passes plus the real fields. NR sweep
    # (the per-voxel model of the constitutive update): read strain 6,
    # plastic strain 6, lambda 6, rho_s 12, rho_m 12, orientation 9; write
    # sigma 6, rho_m 12 -> 69 values of P bytes per voxel.
    alg = {"fwd_z": N * 6 * P + Nh * 6 * 2 * P, "fwd_y": 2 * Nh * 6 * 2 * P,
           "x_green": Nh * 6 * 2 * P + Nh * 9 * 2 * P, "inv_y": 2 * Nh * 9 * 2 * P,
           "inv_z": Nh * 9 * 2 * P + 2 * N * 9 * P,
           "nr": N * NR_ALG_VALUES_PER_VOXEL * P}
    # DRAM bytes per voxel of one launch, from one ncu capture of the kernel
    # (dram__bytes_read.sum + dram__bytes_write.sum on the 96^3 RVE, scaled
    # by voxels)
    traffic_per_voxel = {"nr": NR_DRAM_BYTES_PER_VOXEL}
    for k, b in alg.items():
        if prof[k]["ms_per_launch"]:
            gbs = b / (prof[k]["ms_per_launch"] / 1e3) / 1e9
            prof[k].update({"algorithmic_bytes": b, "achieved_gbs": gbs, "hbm_frac": gbs / hbm})
    pl = prof[dom]
    achieved = alg[dom] / (pl["ms_per_launch"] / 1e3) / 1e9
    traffic = traffic_per_voxel[dom] * N if dom in traffic_per_voxel else None
    newton_per_sweep = newton_prof / (N * it_prof) if it_prof else None
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved,
                "peak": hbm, "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % hbm_src,
                "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg[dom],
                "traffic_over_algorithmic": traffic / alg[dom] if traffic else None}
    if dom == "nr":
        roofline["note"] = ("the NR sweep is bound by the latency of its loads (ncu: long-scoreboard the "
                            "largest stall, 56 %% of DRAM bandwidth, 44 %% of issue slots, 4 blocks of 4 "
                            "warps per SM); its HBM fraction is its distance from the memory roofline at "
                            "%d B/voxel, traffic the bytes its layout moves (per-system constant records)"
                            % (NR_ALG_VALUES_PER_VOXEL * P))
        roofline["newton_steps_per_voxel_sweep"] = newton_per_sweep
        if NR_FP32_FLOP_PER_NEWTON_STEP and newton_per_sweep:
            fl = NR_FP32_FLOP_PER_NEWTON_STEP * newton_per_sweep * N / (pl["ms_per_launch"] / 1e3) / 1e12
            roofline["fp32_pipe"] = {"achieved": fl, "peak": FP32_PEAK_TFLOPS, "unit": "TFLOP/s",
                                     "frac": fl / FP32_PEAK_TFLOPS,
                                     "flop_per_newton_step": NR_FP32_FLOP_PER_NEWTON_STEP,
                                     "peak_source": FP32_PEAK_SOURCE}

    if rank == 0:
        cpu = None
        try:
            with tempfile.TemporaryDirectory(dir=a.workdir) as d:
                case = make_workload(a, d)
                threads = os.cpu_count() or 1
                times = cpu_sample(case, 2, threads)
            cpu = {"value": N * 2 / sum(times), "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": "2 equilibrium iterations of increment 0 of the same %d^3 RVE "
                             "(line-search NR; FFT is the project's CPU DFT, not FFTW)" % a.grid}
        except Exception as e:  # the baseline must not hide the GPU number
            cpu = {"value": None, "unit": UNIT, "cores": None, "kind": "port", "sample": str(e)}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_inc32, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 BC/norms/state)",
            "data": "synthetic", "config": workload_config(a),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 184,
                    "d2h_bytes_per_step": N * 6 * 8 + 2 * 4 * 1024},
            "gpu_launches": int(nlaunch),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "iterations": {"fp32": iters32, "fp64": iters64},
            "fp64": {"value": value64, "ms_per_increment": ms_inc64, "steps": k64},
            "fp32_over_fp64_per_increment": precision["fp32_over_fp64_per_increment"],
            "fp32_macro_sigma_rel_err": max(macro_err),
            "precision": precision,
            "kernels": prof,
            "kernels_fp64": prof64,
            "autotune": {"fp32": tune32, "fp64": tune64},
        }
        line.update(forms)
        print(json.dumps(line), flush=True)


def precision_series(a):
    """The precision form against the FP64 form on the same RVE, increment by
    increment (both run in lockstep, untimed): iteration counts, macroscopic
    stress and von Mises stress relative errors, and the L2 errors of the
    stress and SSD density fields of the FP32-bulk form."""
    import torch
    from srx_gb300 import build
    build.build()
    from srx_gb300 import evpg
    rows = []
    l2 = (lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y)))
    with tempfile.TemporaryDirectory(dir=a.workdir) as d:
        case = make_workload(a, d)
        with evpg.Job(case["input"], case["rho0"], precision=evpg.FP32_BULK, nr_mode=evpg.NR_LINESEARCH) as j32, \
                evpg.Job(case["input"], case["rho0"], precision=evpg.FP64, nr_mode=evpg.NR_LINESEARCH) as j64:
            variant = list(j32.variant())
            for k in range(a.series):
                i32 = j32.increment(k)
                i64 = j64.increment(k)
                s32, s64 = j32.scalars(), j64.scalars()
                rows.append({
                    "increment": k, "iterations_fp32": i32, "iterations_fp64": i64,
                    "macro_sigma_rel_err": float(np.max(np.abs(s32[7:16] - s64[7:16])) / np.max(np.abs(s64[7:16]))),
                    "svm_rel_err": abs(s32[5] - s64[5]) / abs(s64[5]),
                    "sig_l2": l2(j32.download(evpg.F_SIG6), j64.download(evpg.F_SIG6)),
                    "rho_s_l2": l2(j32.download(evpg.F_RHO_S), j64.download(evpg.F_RHO_S)),
                    "svm_fp64": float(s64[5]), "evm": float(s64[1])})
                print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    torch.cuda.synchronize()
    print(json.dumps({"series": "precision form (FP32-bulk) vs FP64", "config": workload_config(a),
                      "variant": variant, "bounds": {"macro_sigma": 1e-4, "field_l2": 1e-3},
                      "max": {k: max(r[k] for r in rows) for k in
                              ("macro_sigma_rel_err", "svm_rel_err", "sig_l2", "rho_s_l2")},
                      "same_iterations": all(r["iterations_fp32"] == r["iterations_fp64"] for r in rows),
                      "rows": rows}), flush=True)


def main():
    a = parse()
    if a.series > 0:
        precision_series(a)
        return
    ws, rank, local = dist_init()
    if a.impl == "reference":
        reference_arm(a, ws, rank)
    else:
        gpu_arm(a, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
