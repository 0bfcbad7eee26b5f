"""Shared fixtures: the oracle (CPU restatement of the reference, used only as
the checker), golden fixtures made by the reference itself, and case
directories written by ``srx_gb300.rve``."""
from __future__ import annotations

import ctypes as C
import json
import os
import platform
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "libevporacle.so")
ORACLE_BIN = os.path.join(ROOT, "oracle", "_build", "evp_oracle")
X86 = platform.machine() in ("x86_64", "AMD64")
# The oracle's OpenMP threads sleep at barriers instead of spinning: with a
# core taken by another process, spinning threads that wait on a descheduled
# one made a two-second 16^3 run take many minutes.
os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def build_oracle():
    if not (os.path.exists(ORACLE_LIB) and os.path.exists(ORACLE_BIN)):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)


class Oracle:
    """ctypes view of oracle/evp_oracle.h."""

    def __init__(self):
        build_oracle()
        L = C.CDLL(ORACLE_LIB)
        L.evo_open.restype = C.c_void_p
        L.evo_open.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]
        L.evo_close.argtypes = [C.c_void_p]
        L.evo_nvox.argtypes = [C.c_void_p]
        L.evo_set_nr_mode.argtypes = [C.c_void_p, C.c_int]
        L.evo_increment.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)]
        L.evo_run.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_int]
        L.evo_field.restype = C.POINTER(C.c_double)
        L.evo_field.argtypes = [C.c_void_p, C.c_char_p]
        L.evo_update_schmid.argtypes = [C.c_void_p]
        L.evo_update_stress.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.evo_set_threads.argtypes = [C.c_int]
        L.evo_set_gnd.argtypes = [C.c_void_p, C.c_int]
        self.L = L

    def open(self, input_path, rho0=None, nr_mode=0, threads=None):
        err = C.create_string_buffer(512)
        self.L.evo_set_threads(threads or min(16, os.cpu_count() or 1))
        h = self.L.evo_open(input_path.encode(), rho0.encode() if rho0 else None, err, 512)
        if not h:
            raise RuntimeError(err.value.decode())
        self.L.evo_set_nr_mode(h, nr_mode)
        return h

    def field(self, h, name, count):
        p = self.L.evo_field(h, name.encode())
        return np.ctypeslib.as_array(p, shape=(count,))


@pytest.fixture(scope="session")
def oracle():
    return Oracle()


def golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    spec = json.loads(str(z["spec"]))
    return z, spec


def write_spec_case(spec, d, print_every=1):
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden  # noqa: E402
    return make_golden.make_input(spec, str(d), print_every=print_every)


def read_iout_fields(d, step, N):
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden  # noqa: E402
    return make_golden.read_fields(str(d), step, N)


def rel_err(a, b):
    """max |a-b| / max |b| (0 when both are 0)."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / s) if s > 0 else float(np.max(np.abs(a)))


def col_err(a, b):
    """Largest per-column error of two tables, each column normalised by its
    own largest |b| (a column of zeros by 1): small columns (strains ~1e-4
    beside stresses ~1e2 MPa, dipole densities ~1e-10 beside SSD densities
    ~10) are checked at the same relative precision as the large ones."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    assert a.shape == b.shape, (a.shape, b.shape)
    s = np.max(np.abs(b), axis=0)
    s = np.where(s > 0, s, 1.0)
    return float(np.max(np.abs(a - b) / s)) if a.size else 0.0


def read_iters(d):
    return [int(l.split()[1]) for l in open(os.path.join(str(d), "iters.txt")) if l.strip()]


def read_table(p):
    return np.loadtxt(p, skiprows=1, ndmin=2)
