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
                  [--grains 1000] [--fp64-steps K64]

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
UNIT = "voxel-iterations/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    p.add_argument("--grid", type=int, default=128, help="RVE edge length in voxels")
    p.add_argument("--grains", type=int, default=1000)
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--workdir", default=None)
    p.add_argument("--batch-count", type=int, default=64)
    p.add_argument("--batch-steps", type=int, default=2)
    p.add_argument("--serve-requests", type=int, default=24)
    p.add_argument("--serve-rates", default="2,16")
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
    graphs). Host wall time around synchronous calls."""
    from srx_gb300 import workloads
    cases = workloads.batch_set(os.path.join(root, "batch"), count=a.batch_count, steps=a.batch_steps)
    nsteps = [a.batch_steps] * len(cases)
    out = {"rves": len(cases), "increments_per_rve": a.batch_steps,
           "grids": sorted(set(c["n"] for c in cases)), "voxels": int(sum(c["N"] for c in cases)),
           "loads": {k: sum(1 for c in cases if c["load"] == k) for k in ("tension", "compression", "shear")}}
    for prec, tag in ((evpg.FP32_BULK, "fp32"), (evpg.FP64, "fp64")):
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
        rec = {"value": vi / tb, "unit": UNIT, "seconds": tb, "rounds": rounds,
               "iterations": int(sum(sum(i) for i in its))}
        if tag == "fp32":
            jobs = [evpg.Job(c["input"], c["rho0"], precision=prec, nr_mode=evpg.NR_LINESEARCH) for c in cases]
            for j in jobs:
                if not a.no_tune:
                    j.tune()
            t0 = time.perf_counter()
            its_alone = [[j.increment(k) for k in range(a.batch_steps)] for j in jobs]
            ta = time.perf_counter() - t0
            for j in jobs:
                j.close()
            rec["alone_sequential"] = {"value": vi / ta, "seconds": ta,
                                       "same_iterations": its_alone == its}
            rec["batch_over_alone"] = ta / tb
        out[tag] = rec
    return out


def serve_leg(a, evpg, root, budget):
    """Serving form: Poisson request streams through the continuous-batching
    server (FP32-bulk); latency per solve and per increment, solves/s."""
    from srx_gb300 import workloads
    rates = [float(r) for r in a.serve_rates.split(",") if r]
    base = workloads.serve_stream(os.path.join(root, "serve"), count=a.serve_requests, rate_hz=1.0,
                                  steps=(2, 4), distinct=min(12, a.serve_requests))
    out = {"requests": len(base), "grids": sorted(set(c["n"] for c in base)),
           "increments_per_request": [2, 4], "rates": {}}
    for rate in rates:
        with evpg.Server(precision=evpg.FP32_BULK, nr_mode=evpg.NR_LINESEARCH, hbm_budget=budget,
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
        out["rates"][str(rate)] = {
            "solves_per_s": st.solves_per_s, "solve_p50_s": st.solve_p50, "solve_p99_s": st.solve_p99,
            "increment_p50_s": st.incr_p50, "increment_p99_s": st.incr_p99,
            "completed": st.completed, "failed": st.failed, "rounds": st.rounds,
            "iterations": int(st.iterations), "span_s": st.span}
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
        tune32 = {"gain": None if a.no_tune else j32.tune(), "schedule": j32.schedule()}
        for s in range(a.warmup):
            j32.increment(s)
        barrier(ws)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        iters32, sig32 = [], []
        l0 = launches(j32)
        with Clocks(local) as clk:
            ev0.record(stream)
            for s in range(a.warmup, a.warmup + a.steps):
                iters32.append(j32.increment(s))
                sig32.append(j32.scalars()[7:16].copy())
            ev1.record(stream)
            torch.cuda.synchronize()
        nlaunch = launches(j32) - l0
        t32 = ev0.elapsed_time(ev1) / 1e3
        clocks = clk.summary()
        barrier(ws)
        tmax = allmax(ws, t32)
        vi = allsum(ws, float(N * sum(iters32)))
        value = vi / tmax

        # ---------------- e2e through the C ABI with host buffers
        host = np.empty((N, 6), dtype=np.float64)
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
        del host

        # ---------------- per-kernel times (profiling run, one increment)
        prof = {}
        evpg.check(L.evpg_profile(j32.ctx, 1))
        s_prof = s0 + a.e2e_steps
        it_prof = j32.increment(s_prof)
        ms = (C.c_double * 10)()
        nl = (C.c_int64 * 10)()
        evpg.check(L.evpg_profile_read(j32.ctx, ms, nl, 10))
        evpg.check(L.evpg_profile(j32.ctx, 0))
        names = ["fwd_z", "fwd_y", "x_green", "inv_y", "inv_z", "nr", "macro", "begin", "end",
                 "refine"]
        for i, nm in enumerate(names):
            prof[nm] = {"ms_total": ms[i], "launches": int(nl[i]),
                        "ms_per_launch": ms[i] / nl[i] if nl[i] else None}
        j32.close()

        # ---------------- FP64 plain form on the same increments
        j64 = open_job(evpg.FP64)
        tune64 = {"gain": None if a.no_tune else j64.tune(), "schedule": j64.schedule()}
        for s in range(a.warmup):
            j64.increment(s)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        iters64, sig64 = [], []
        e0.record(stream)
        for s in range(a.warmup, a.warmup + min(a.fp64_steps, a.steps)):
            iters64.append(j64.increment(s))
            sig64.append(j64.scalars()[7:16].copy())
        e1.record(stream)
        torch.cuda.synchronize()
        t64 = e0.elapsed_time(e1) / 1e3
        j64.close()

        forms = {}
        wanted = [f for f in a.forms.split(",") if f]
        if "batch" in wanted:
            forms["batching"] = batch_leg(a, evpg, d)
        if "serve" in wanted:
            free, _ = torch.cuda.mem_get_info()
            forms["serving"] = serve_leg(a, evpg, d, int(0.8 * free))

    k64 = len(iters64)
    value64 = N * sum(iters64) / t64
    ms_inc32 = 1e3 * t32 / a.steps
    ms_inc64 = 1e3 * t64 / k64
    macro_err = max(float(np.max(np.abs(sig32[i] - sig64[i])) / np.max(np.abs(sig64[i])))
                    for i in range(k64))

    # roofline of the dominant kernel group (by time in the profiling run)
    dom = max(("fwd_z", "fwd_y", "x_green", "inv_y", "inv_z", "nr"), key=lambda k: prof[k]["ms_total"])
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    Nh = a.grid * a.grid * (a.grid // 2 + 1)
    # algorithmic HBM bytes per launch (FP32 bulk). NR per voxel: reads
    # lambda 6, strain 6, Eps - eps_begin 6, Schmid 60, flow constants 36
    # (FP32), orientation and phase ids 8 B; writes sigma 6.
    alg = {"fwd_z": N * 6 * 4 + Nh * 6 * 8, "fwd_y": 2 * Nh * 6 * 8,
           "x_green": Nh * 6 * 8 + Nh * 9 * 8, "inv_y": 2 * Nh * 9 * 8,
           "inv_z": Nh * 9 * 8 + 2 * N * 9 * 4,
           "nr": N * ((6 + 6 + 6 + 60 + 36 + 6) * 4 + 8)}
    # DRAM bytes per voxel of one launch, from one ncu capture of the kernel
    # (dram__bytes_read.sum + dram__bytes_write.sum on the 96^3 RVE, scaled
    # by voxels; profiles/k_nr_fp32_96cube.md)
    traffic_per_voxel = {"nr": NR_DRAM_BYTES_PER_VOXEL}
    for k, b in alg.items():
        if prof[k]["ms_per_launch"]:
            gbs = b / (prof[k]["ms_per_launch"] / 1e3) / 1e9
            prof[k].update({"algorithmic_bytes": b, "achieved_gbs": gbs, "hbm_frac": gbs / hbm})
    pl = prof[dom]
    achieved = alg[dom] / (pl["ms_per_launch"] / 1e3) / 1e9
    traffic = traffic_per_voxel[dom] * N if dom in traffic_per_voxel else None
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved,
                "peak": hbm, "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)",
                "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg[dom],
                "note": "the NR sweep is issue-bound (FP32 pipe), not HBM-bound: its DRAM traffic "
                        "equals its algorithmic bytes, so the HBM fraction is its distance from "
                        "the memory roofline"}

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
            "fp32_over_fp64_per_increment": ms_inc64 / ms_inc32,
            "fp32_macro_sigma_rel_err": macro_err,
            "kernels": prof,
            "autotune": {"fp32": tune32, "fp64": tune64},
        }
        line.update(forms)
        print(json.dumps(line), flush=True)


def main():
    a = parse()
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
