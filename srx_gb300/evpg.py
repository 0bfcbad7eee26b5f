"""ctypes binding of the C ABI in ``include/evpg.h``.

The CUDA library ``srx_gb300/_lib/libevpg.so`` is the only compute path;
importing this module fails when it is missing (call
``srx_gb300.build.build()`` first). There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import build as _build

EVPG_OK = 0
FP64, FP32_BULK = 0, 1
NR_PLAIN, NR_LINESEARCH = 0, 1
F_SIG, F_DISGRAD, F_EPS, F_EDOT, F_TRANMAT = 0, 1, 2, 3, 4
F_RHO_S, F_RHO_M, F_GAMDOT, F_GAM_ACUM, F_VELGRAD, F_SIG6 = 5, 6, 7, 8, 9, 10
F_RHO_G1, F_RHO_G2 = 11, 12  # GND densities (jobs opened with gnd=True)
FIELD_WIDTH = {F_SIG: 9, F_DISGRAD: 9, F_EPS: 9, F_EDOT: 9, F_TRANMAT: 9, F_RHO_S: 12,
               F_RHO_M: 12, F_GAMDOT: 12, F_GAM_ACUM: 12, F_VELGRAD: 9, F_SIG6: 6,
               F_RHO_G1: 12, F_RHO_G2: 12}
JOB_GND = 1  # evpg_job_open_opts option: first-order GND densities (DD_GND)


class EvpgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("evpg status %d: %s" % (status, msg))
        self.status = status


class IterOut(C.Structure):
    _fields_ = [("err_e", C.c_double), ("err_s", C.c_double), ("err_e_sum", C.c_double),
                ("err_s_sum", C.c_double), ("sig_avg", C.c_double * 9),
                ("sig_avg_ph1", C.c_double * 9), ("ddisgrad", C.c_double * 9),
                ("ddisgrad_acum", C.c_double * 9), ("s_vm", C.c_double), ("s_vm1", C.c_double),
                ("iter", C.c_int32), ("converged", C.c_int32)]


class IncrOut(C.Structure):
    _fields_ = [("eps_avg", C.c_double * 9), ("edot_avg", C.c_double * 9),
                ("rho_avg", C.c_double * 8), ("nr_iterations", C.c_int64)]


_LIB = None


def lib() -> C.CDLL:
    """The loaded CUDA library (RuntimeError when it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(_build.LIB):
            raise RuntimeError("libevpg.so is not built: run srx_gb300.build.build() (nvcc, sm_103a)")
        L = C.CDLL(_build.LIB)
        vp, i32, d, sz = C.c_void_p, C.c_int32, C.c_double, C.c_size_t
        L.evpg_version.restype = C.c_char_p
        L.evpg_last_error.restype = C.c_char_p
        L.evpg_status_string.restype = C.c_char_p
        L.evpg_status_string.argtypes = [C.c_int]
        L.evpg_job_open.argtypes = [C.c_char_p, C.c_char_p, i32, i32, C.POINTER(vp)]
        L.evpg_job_open_opts.argtypes = [C.c_char_p, C.c_char_p, i32, i32, i32, C.POINTER(vp)]
        L.evpg_job_close.argtypes = [vp]
        L.evpg_job_ctx.argtypes = [vp]
        L.evpg_job_ctx.restype = vp
        L.evpg_job_nvox.argtypes = [vp, C.POINTER(i32)]
        L.evpg_job_nsteps.argtypes = [vp]
        L.evpg_job_increment.argtypes = [vp, i32, C.POINTER(i32)]
        L.evpg_job_scalars.argtypes = [vp, C.POINTER(d), i32]
        L.evpg_job_run.argtypes = [vp, C.c_char_p, i32, i32]
        L.evpg_download.argtypes = [vp, i32, C.POINTER(d), sz]
        L.evpg_upload.argtypes = [vp, i32, C.POINTER(d), sz]
        L.evpg_equilibrium_iteration.argtypes = [vp, d, C.POINTER(IterOut)]
        L.evpg_equilibrium_solve.argtypes = [vp, d, C.POINTER(IterOut)]
        L.evpg_increment_begin.argtypes = [vp, C.POINTER(d), i32, C.POINTER(d), d]
        L.evpg_increment_end.argtypes = [vp, i32, C.POINTER(IncrOut)]
        L.evpg_synchronize.argtypes = [vp]
        L.evpg_device_bytes.argtypes = [vp, C.POINTER(C.c_int64)]
        L.evpg_launch_count.argtypes = [vp, C.POINTER(C.c_int64)]
        L.evpg_set_stream.argtypes = [vp, vp]
        L.evpg_increment.argtypes = [vp, C.POINTER(d), i32, C.POINTER(d), d, d, i32,
                                     C.POINTER(IterOut), C.POINTER(IncrOut)]
        L.evpg_batch_create.argtypes = [i32, i32, C.POINTER(vp)]
        L.evpg_batch_destroy.argtypes = [vp]
        L.evpg_batch_set.argtypes = [vp, C.POINTER(vp), i32]
        L.evpg_batch_stage.argtypes = [vp, i32, C.POINTER(d), i32, C.POINTER(d), d, d, i32]
        L.evpg_batch_round.argtypes = [vp, i32, C.POINTER(i32)]
        L.evpg_batch_slot.argtypes = [vp, i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(IterOut),
                                      C.POINTER(IncrOut)]
        L.evpg_batch_launch_count.argtypes = [vp, C.POINTER(C.c_int64)]
        L.evpg_job_stage.argtypes = [vp, vp, i32, i32]
        L.evpg_job_collect.argtypes = [vp, vp, i32, C.POINTER(i32), C.POINTER(i32)]
        L.evpg_jobs_run_batched.argtypes = [C.POINTER(vp), i32, C.POINTER(i32), i32, C.POINTER(i32),
                                            i32, C.POINTER(C.c_int64)]
        _LIB = L
    return _LIB


def check(st: int) -> None:
    if st != EVPG_OK:
        L = lib()
        raise EvpgError(st, "%s: %s" % (L.evpg_status_string(st).decode(),
                                        L.evpg_last_error().decode()))


class Job:
    """A job of the host driver: the reference's input files on the device.
    gnd=True adds the first-order GND densities (the reference built with
    DD_GND)."""

    def __init__(self, input_path: str, rho0: Optional[str] = None, precision: int = FP64,
                 nr_mode: int = NR_PLAIN, gnd: bool = False):
        L = lib()
        h = C.c_void_p()
        check(L.evpg_job_open_opts(input_path.encode(), rho0.encode() if rho0 else None,
                                   precision, nr_mode, JOB_GND if gnd else 0, C.byref(h)))
        self._h = h
        n = (C.c_int32 * 3)()
        check(L.evpg_job_nvox(h, n))
        self.n = tuple(n)
        self.N = n[0] * n[1] * n[2]
        self.precision = precision

    @property
    def ctx(self) -> C.c_void_p:
        return C.c_void_p(lib().evpg_job_ctx(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().evpg_job_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def n_steps(self) -> int:
        return lib().evpg_job_nsteps(self._h)

    def increment(self, istep: int) -> int:
        it = C.c_int32()
        check(lib().evpg_job_increment(self._h, istep, C.byref(it)))
        return it.value

    def scalars(self) -> np.ndarray:
        out = (C.c_double * 34)()
        check(lib().evpg_job_scalars(self._h, out, 34))
        return np.array(out[:])

    def run(self, outdir: str, nsteps: int = -1, iout: bool = False) -> None:
        check(lib().evpg_job_run(self._h, outdir.encode(), nsteps, 1 if iout else 0))

    def download(self, field: int) -> np.ndarray:
        w = FIELD_WIDTH[field]
        out = np.empty(self.N * w, dtype=np.float64)
        check(lib().evpg_download(self.ctx, field, out.ctypes.data_as(C.POINTER(C.c_double)),
                                  out.size))
        return out.reshape(self.N, w)

    def download_into(self, field: int, out: np.ndarray) -> np.ndarray:
        """Download into a caller's C-contiguous float64 array (pinned memory
        is written directly by the copy engine)."""
        w = FIELD_WIDTH[field]
        if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.size < self.N * w:
            raise ValueError("need a C-contiguous float64 array of %d values" % (self.N * w))
        check(lib().evpg_download(self.ctx, field, out.ctypes.data_as(C.POINTER(C.c_double)),
                                  out.size))
        return out

    def upload(self, field: int, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
        check(lib().evpg_upload(self.ctx, field, a.ctypes.data_as(C.POINTER(C.c_double)), a.size))

    def device_bytes(self) -> int:
        b = C.c_int64()
        check(lib().evpg_device_bytes(self.ctx, C.byref(b)))
        return b.value

    def launches(self) -> int:
        n = C.c_int64()
        check(lib().evpg_launch_count(self.ctx, C.byref(n)))
        return n.value

    def tune(self, force: bool = False) -> float:
        """Autotune the spectral schedule; returns default/tuned time (0 if cached)."""
        lib().evpg_tune.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]
        g = C.c_double()
        check(lib().evpg_tune(self.ctx, 1 if force else 0, C.byref(g)))
        return g.value

    def set_fused(self, mode: int) -> None:
        """Fused z+y passes: -1 default, 0 off, 1 on where eligible."""
        lib().evpg_set_fused.argtypes = [C.c_void_p, C.c_int32]
        check(lib().evpg_set_fused(self.ctx, mode))

    def set_xpass(self, mode: int) -> None:
        """Warp-register X pass: -1 default, 0 shared-memory pass, 1 on where eligible."""
        lib().evpg_set_xpass.argtypes = [C.c_void_p, C.c_int32]
        check(lib().evpg_set_xpass(self.ctx, mode))

    def set_radix(self, axis: int, radices) -> None:
        """FFT radix order of one axis (0 x, 1 y, 2 z) for the Stockham passes."""
        L = lib()
        L.evpg_set_radix.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.c_int32]
        arr = (C.c_int32 * len(radices))(*radices)
        check(L.evpg_set_radix(self.ctx, axis, arr, len(radices)))

    def schedule(self) -> dict:
        """Pencils per CTA (z, y, x passes) and radix stages (x, y, z axes)."""
        lib().evpg_get_schedule.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                            C.POINTER(C.c_int32)]
        P = (C.c_int32 * 3)()
        R = (C.c_int32 * 36)()
        S = (C.c_int32 * 3)()
        check(lib().evpg_get_schedule(self.ctx, P, R, S))
        return {"pencils_zyx": list(P), "radix_xyz": [list(R[12 * a:12 * a + S[a]]) for a in range(3)]}

    def variant(self) -> tuple:
        """(plane-kernel values per lane, warp X-pass values per lane); 0 means
        the separate Stockham passes run instead."""
        lib().evpg_get_variant.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        v = (C.c_int32 * 2)()
        check(lib().evpg_get_variant(self.ctx, v))
        return (v[0], v[1])

    def set_load_from(self, input_path: str) -> None:
        """Switch to the boundary conditions of another namelist."""
        lib().evpg_job_set_load_from.argtypes = [C.c_void_p, C.c_char_p]
        check(lib().evpg_job_set_load_from(self._h, input_path.encode()))


def run_batched(jobs, nsteps, max_ticks: int = 16):
    """Advance ``nsteps[i]`` increments of every job in one batch (rounds of
    at most ``max_ticks`` equilibrium iterations). Returns the per-increment
    iteration counts (list of lists) and the number of rounds."""
    n = len(jobs)
    stride = max(nsteps) if nsteps else 1
    hs = (C.c_void_p * n)(*[j._h for j in jobs])
    ns = (C.c_int32 * n)(*nsteps)
    it = (C.c_int32 * (n * stride))()
    rounds = C.c_int64()
    check(lib().evpg_jobs_run_batched(hs, n, ns, max_ticks, it, stride, C.byref(rounds)))
    return [list(it[i * stride:i * stride + nsteps[i]]) for i in range(n)], rounds.value


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("increments", C.c_int32),
                ("iterations", C.c_int64), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("device_bytes", C.c_int64)]


class ServeStats(C.Structure):
    _fields_ = [("completed", C.c_int32), ("failed", C.c_int32), ("increments", C.c_int64),
                ("iterations", C.c_int64), ("rounds", C.c_int64), ("ticks", C.c_int64),
                ("solve_p50", C.c_double), ("solve_p99", C.c_double), ("incr_p50", C.c_double),
                ("incr_p99", C.c_double), ("span", C.c_double), ("solves_per_s", C.c_double)]


class ServerCfg(C.Structure):
    _fields_ = [("precision", C.c_int32), ("nr_mode", C.c_int32), ("hbm_budget", C.c_int64),
                ("max_slots", C.c_int32), ("round_ticks", C.c_int32), ("loaders", C.c_int32),
                ("keep_fields", C.c_int32), ("job_options", C.c_int32)]


class Server:
    """Continuous-batching server of ``include/evpg.h`` (evpg_server_*)."""

    def __init__(self, precision: int = FP32_BULK, nr_mode: int = NR_LINESEARCH,
                 hbm_budget: int = 64 << 30, max_slots: int = 64, round_ticks: int = 16,
                 loaders: int = 4, keep_fields: bool = False, gnd: bool = False):
        L = lib()
        vp = C.c_void_p
        L.evpg_server_create.argtypes = [C.POINTER(ServerCfg), C.POINTER(vp)]
        L.evpg_server_submit.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_int32, C.c_int32, C.c_char_p,
                                         C.POINTER(C.c_int64)]
        L.evpg_server_wait.argtypes = [vp, C.c_double]
        L.evpg_server_request.argtypes = [vp, C.c_int64, C.POINTER(RequestInfo)]
        L.evpg_server_stats.argtypes = [vp, C.POINTER(ServeStats)]
        L.evpg_server_result.argtypes = [vp, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.c_size_t, C.POINTER(C.c_double)]
        L.evpg_server_destroy.argtypes = [vp]
        cfg = ServerCfg(precision, nr_mode, hbm_budget, max_slots, round_ticks, loaders,
                        1 if keep_fields else 0, JOB_GND if gnd else 0)
        h = C.c_void_p()
        check(L.evpg_server_create(C.byref(cfg), C.byref(h)))
        self._h = h

    def submit(self, input_path: str, nsteps: int, rho0: Optional[str] = None,
               switch_step: int = -1, switch_input: Optional[str] = None) -> int:
        rid = C.c_int64()
        check(lib().evpg_server_submit(self._h, input_path.encode(), rho0.encode() if rho0 else None,
                                       nsteps, switch_step,
                                       switch_input.encode() if switch_input else None, C.byref(rid)))
        return rid.value

    def wait(self, timeout_s: float = 3600.0) -> None:
        check(lib().evpg_server_wait(self._h, timeout_s))

    def request(self, rid: int) -> RequestInfo:
        info = RequestInfo()
        check(lib().evpg_server_request(self._h, rid, C.byref(info)))
        return info

    def stats(self) -> ServeStats:
        s = ServeStats()
        check(lib().evpg_server_stats(self._h, C.byref(s)))
        return s

    def result(self, rid: int, nvox: int):
        sig = np.empty(6 * nvox)
        rho = np.empty(12 * nvox)
        sc = np.empty(34)
        dp = C.POINTER(C.c_double)
        check(lib().evpg_server_result(self._h, rid, sig.ctypes.data_as(dp), rho.ctypes.data_as(dp),
                                       nvox, sc.ctypes.data_as(dp)))
        return sig.reshape(nvox, 6), rho.reshape(nvox, 12), sc

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().evpg_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
