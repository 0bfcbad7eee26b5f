"""The C-ABI library builds for sm_103a, loads, exports every entry point of
include/evpg.h, and refuses to run without a GPU (no CPU fallback)."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "evpg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(evpg_\w+)\s*\(", src, re.M)))


def test_header_declares_entry_points():
    names = _declared()
    for n in ("evpg_create", "evpg_destroy", "evpg_increment_begin", "evpg_equilibrium_iteration",
              "evpg_equilibrium_solve", "evpg_increment_end", "evpg_download", "evpg_job_open",
              "evpg_job_run"):
        assert n in names


def test_library_builds_and_exports_every_symbol():
    from srx_gb300 import build
    path = build.build()
    lib = C.CDLL(path)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert os.path.exists(build.RUN)


def test_header_compiles_as_c_with_struct_tags(tmp_path):
    """A C caller may name every structure of the header by its tag
    (struct evpg_x) or by its typedef (evpg_x): each typedef's tag is its
    own name."""
    import subprocess
    src = open(os.path.join(ROOT, "include", "evpg.h")).read()
    tags, names = [], []
    for m in re.finditer(r"typedef\s+struct\s+(\w+)\s*\{", src):
        tags.append(m.group(1))
        names.append(re.compile(r"\}\s*(\w+)\s*;").search(src, m.end()).group(1))
    assert tags and tags == names, list(zip(tags, names))
    c = tmp_path / "use.c"
    c.write_text('#include "evpg.h"\n' + "".join(
        "struct %s a%d; %s b%d;\n" % (t, i, t, i) for i, t in enumerate(tags)) +
        "int main(void) { return 0; }\n")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-c", str(c), "-o", str(tmp_path / "use.o")], check=True)


def test_no_cpu_fallback_without_device(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from srx_gb300 import evpg, rve
    case = rve.make_case(str(tmp_path / "c"), (8, 8, 8), 3, 1, rve.Job(n=(8, 8, 8), n_steps=1))
    with pytest.raises(evpg.EvpgError) as e:
        evpg.Job(case["input"])
    assert e.value.status == 9  # EVPG_ERR_NO_DEVICE


def test_namelist_parsing_is_thread_safe(tmp_path):
    """The server's loader threads parse namelists concurrently: many threads
    reading different files get their own grids (no shared tokenizer state)."""
    import ctypes as C
    import threading
    from srx_gb300 import evpg, rve
    L = evpg.lib()
    L.evpg_job_grid.argtypes = [C.c_char_p, C.POINTER(C.c_int32)]
    paths = []
    for i in range(12):
        n = (8 + i, 9 + 2 * i, 10 + 3 * i)
        p = str(tmp_path / ("input%d" % i))
        rve.write_namelist(p, rve.Job(n=n, load=["tension", "shear"][i % 2]), rve.Material(), "ms.txt", "cu.sx")
        paths.append((p, n))
    bad = []

    def worker(k):
        out = (C.c_int32 * 3)()
        for r in range(200):
            p, n = paths[(k + r) % len(paths)]
            if L.evpg_job_grid(p.encode(), out) != 0 or tuple(out) != n:
                bad.append((p, tuple(out), n))
    ts = [threading.Thread(target=worker, args=(k,)) for k in range(8)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not bad, bad[:3]
