"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs the reference's own sources compiled with single-rank shims
(oracle/_ref/srx_ref, srx_ref_nrmod and srx_ref_gnd, built by ``make -C oracle
ref`` from the reference tree) on small cases and stores what it writes:

* ``bicrystal8``   the reference's 8^3 regression case (restated by
                   ``srx_gb300.rve.bicrystal8_case``), plain NR, 10 increments:
                   vm.out, dd.out, per-increment iteration counts and the
                   .iout fields (stress, plastic strain, per-system SSD density,
                   accumulated slip, texture) at increments 0, 1, 2, 4, 9;
* ``voronoi16_ls`` 16^3, 8 Voronoi grains, benchmark material, z tension,
                   NR_MODIFIED line search, 2 increments, full final fields;
* ``cfg0_32_ls``   the 32^3 / 27-grain configuration, line search, first
                   increment, fields on every 7th voxel;
* ``gnd12_ls``     12^3, 6 Voronoi grains, line search with first-order GND
                   densities (srx_ref_gnd: DD_GND), 5 increments -- the slip-rate
                   gradients start in the third increment (istep > 1) and reach
                   the flow rule in the fourth; full final fields including
                   the GND densities;
* ``cfg0_32_run``  the 32^3 / 27-grain configuration over all 50 increments:
                   iteration counts, vm.out and dd.out of every increment,
                   fields at increments 0, 14, 28, 49 on every 7th voxel;
* ``cfg1_64_ls``   the 64^3 / 125-grain configuration, first 5 increments,
                   fields at increments 0 and 4 on every 31st voxel;
* ``cfg2_128_ls``  the 128^3 / 1000-grain precision-form configuration with
                   per-grain log-uniform initial density (the benchmark's RVE),
                   first 2 increments, fields of both on every 251st voxel;
* ``setup16``      the set-up state of ``voronoi16_ls`` (C066, S066, Schmid
                   tensors, interaction matrices, shear modulus, Burgers length);
* ``nrprobe8``     one UpdateStress sweep of the reference on the bicrystal
                   state with a perturbed displacement gradient.

Usage: python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from srx_gb300 import rve  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "srx_ref")
REF_LS = os.path.join(ROOT, "oracle", "_ref", "srx_ref_nrmod")
REF_GND = os.path.join(ROOT, "oracle", "_ref", "srx_ref_gnd")

# .iout component order 11,22,33,23,13,12 (io.c:409-421)


def voronoi16_spec():
    return dict(kind="voronoi", n=[16, 16, 16], grains=8, seed=1008, steps=2, nr="ls",
                rho0=None)


def cfg0_32_spec():
    return dict(kind="voronoi", n=[32, 32, 32], grains=27, seed=1027, steps=1, nr="ls",
                rho0=None)


def gnd12_spec():
    return dict(kind="voronoi", n=[12, 12, 12], grains=6, seed=1212, steps=5, nr="ls",
                rho0=None, gnd=True)


def cfg0_32_run_spec():
    """The 32^3 / 27-grain configuration over its whole load path (50
    increments of 2e-4 strain)."""
    return dict(kind="voronoi", n=[32, 32, 32], grains=27, seed=1027, steps=50, nr="ls",
                rho0=None, keep=[0, 14, 28, 49], print_every=7, stride=7)


def cfg1_64_spec():
    """The 64^3 / 125-grain configuration, first five increments."""
    return dict(kind="voronoi", n=[64, 64, 64], grains=125, seed=1125, steps=5, nr="ls",
                rho0=None, keep=[0, 4], print_every=2, stride=31)


def cfg2_128_spec():
    """The 128^3 / 1000-grain precision-form configuration (per-grain initial
    density log-uniform in [5e11, 5e12] m^-2, seed 2025: the benchmark's own
    RVE), first two increments."""
    return dict(kind="voronoi", n=[128, 128, 128], grains=1000, seed=2025, steps=2, nr="ls",
                rho0=[0.5, 5.0], keep=[0, 1], print_every=1, stride=251)


def make_input(spec: dict, d: str, print_every: int = 1) -> dict:
    """Write the case directory of a spec (shared with the tests)."""
    if spec["kind"] == "bicrystal8":
        return rve.bicrystal8_case(d, n_steps=spec["steps"], print_every=print_every)
    job = rve.Job(n=tuple(spec["n"]), n_steps=spec["steps"], print_control=(1, print_every))
    return rve.make_case(d, spec["n"], spec["grains"], spec["seed"], job,
                         rho0=spec.get("rho0"))


def run_ref(binary: str, case: dict, extra=()):
    args = [binary, "input"] + list(extra)
    if case.get("rho0"):
        args += ["--rho0", os.path.basename(case["rho0"])]
    r = subprocess.run(args, cwd=case["dir"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference failed (%d): %s" % (r.returncode, r.stdout[-2000:]))
    iters, errs, cnt = [], [], 0
    for line in r.stdout.splitlines():
        if line.startswith("STEP ="):
            if cnt or iters or errs:
                iters.append(cnt)
            cnt = 0
        elif line.startswith("Strain field error"):
            cnt += 1
    iters.append(cnt)
    return iters


def read_table(p):
    return np.loadtxt(p, skiprows=1, ndmin=2)


def read_fields(d: str, step: int, N: int) -> dict:
    f = {}
    f["sig"] = np.stack([np.fromfile(os.path.join(d, "sig_afterDRX_%d_S%06d.iout" % (c + 1, step)))
                         for c in range(6)], axis=1)
    f["eps"] = np.stack([np.fromfile(os.path.join(d, "eps_%d_S%06d.iout" % (c + 1, step)))
                         for c in range(6)], axis=1)
    f["els"] = np.stack([np.fromfile(os.path.join(d, "els_%d_S%06d.iout" % (c + 1, step)))
                         for c in range(6)], axis=1)
    rec = np.fromfile(os.path.join(d, "dislocation_afterDRX_S%04d.iout" % step), dtype=np.uint8)
    f["rho_s"] = rec.reshape(N, 104)[:, 8:].copy().view(np.float64)
    rec = np.fromfile(os.path.join(d, "slip_afterDRX_S%04d.iout" % step), dtype=np.uint8)
    f["gam_acum"] = rec.reshape(N, 104)[:, 8:].copy().view(np.float64)
    rec = np.fromfile(os.path.join(d, "tex_afterDRX_S%06d.iout" % step), dtype=np.uint8)
    f["tex"] = rec.reshape(N, 48)[:, :24].copy().view(np.float64)
    f["newpos"] = np.fromfile(os.path.join(d, "new_position_afterDRX_S%04d.iout" % step)).reshape(N, 3)
    return f


def gen_bicrystal8(out: str) -> None:
    spec = dict(kind="bicrystal8", steps=10, nr="plain")
    keep = [0, 1, 2, 4, 9]
    with tempfile.TemporaryDirectory() as t:
        case = make_input(spec, t)
        iters = run_ref(REF, case)
        data = {"iters": np.array(iters), "vm": read_table(os.path.join(t, "vm.out")),
                "dd": read_table(os.path.join(t, "dd.out")), "keep": np.array(keep)}
        for s in keep:
            for k, v in read_fields(t, s, 512).items():
                data["%s_%d" % (k, s)] = v
    np.savez_compressed(out, spec=json.dumps(spec), **data)


def gen_voronoi(spec: dict, out: str, stride: int = 1) -> None:
    with tempfile.TemporaryDirectory() as t:
        case = make_input(spec, t)
        binary = REF_GND if spec.get("gnd") else (REF_LS if spec["nr"] == "ls" else REF)
        iters = run_ref(binary, case, ["--final", "final.bin"])
        N = int(np.prod(spec["n"]))
        last = spec["steps"] - 1
        f = read_fields(t, last, N)
        idx = np.arange(0, N, stride)
        data = {"iters": np.array(iters), "vm": read_table(os.path.join(t, "vm.out")),
                "dd": read_table(os.path.join(t, "dd.out")), "idx": idx}
        for k, v in f.items():
            data[k] = v[idx]
        fin = final_state(os.path.join(t, "final.bin"))
        keys = ["rho_m", "gamdot", "TranMat", "DisGrad", "Edot"]
        if spec.get("gnd"):
            keys += ["Sig", "rho_s", "rho_g1", "rho_g2"]
        for k in keys:
            data["final_" + k] = fin[k][idx]
    np.savez_compressed(out, spec=json.dumps(spec), **data)


def gen_run(spec: dict, out: str) -> None:
    """A multi-increment run: iteration counts, vm.out and dd.out of every
    increment, and the .iout fields of the increments in spec["keep"] on every
    spec["stride"]-th voxel (keys "<field>_<increment>")."""
    with tempfile.TemporaryDirectory() as t:
        case = make_input(spec, t, print_every=spec["print_every"])
        iters = run_ref(REF_LS, case)
        N = int(np.prod(spec["n"]))
        idx = np.arange(0, N, spec["stride"])
        data = {"iters": np.array(iters), "vm": read_table(os.path.join(t, "vm.out")),
                "dd": read_table(os.path.join(t, "dd.out")), "idx": idx,
                "keep": np.array(spec["keep"])}
        for s in spec["keep"]:
            for k, v in read_fields(t, s, N).items():
                if k in RUN_FIELDS:
                    data["%s_%d" % (k, s)] = v[idx]
    np.savez_compressed(out, spec=json.dumps(spec), **data)


# fields a multi-increment fixture keeps (stress, SSD density, accumulated slip)
RUN_FIELDS = ("sig", "rho_s", "gam_acum")


def final_state(p: str) -> dict:
    b = open(p, "rb").read()
    N, ns = np.frombuffer(b[:8], dtype=np.int32)
    off = 8
    out = {}

    def take(name, n):
        nonlocal off
        out[name] = np.frombuffer(b[off:off + 8 * n]).copy()
        off += 8 * n

    for k in ("Sig", "DisGrad", "Eps", "Edot", "VelGrad", "TranMat"):
        take(k, 9 * N)
        out[k] = out[k].reshape(N, 9)
    for k in ("rho_s", "rho_m", "rho_F", "rho_P", "gamdot", "gam_acum", "trial_gam_acum",
              "rho_dipole", "rho_forest", "rho_inplane"):
        take(k, 12 * N)
        out[k] = out[k].reshape(N, 12)
    take("rho_tot", N)
    off += 8 * (4 * 9 + 13)  # SigAvg, SigAvg1, dDisGradAvg_acum, DisGradAvg, scalars
    if len(b) >= off + 3 * 8 * 12 * N:  # GND densities (harness builds that dump them)
        for k in ("rho_g1", "rho_g2", "rho_g3"):
            take(k, 12 * N)
            out[k] = out[k].reshape(N, 12)
    return out


def gen_setup16(out: str) -> None:
    spec = voronoi16_spec()
    with tempfile.TemporaryDirectory() as t:
        case = make_input(spec, t)
        subprocess.run([REF, "input", "--setup", "setup.bin"], cwd=t, capture_output=True,
                       check=True)
        b = open(os.path.join(t, "setup.bin"), "rb").read()
    N = int(np.prod(spec["n"]))
    off = 8
    data = {}

    def take(name, n):
        nonlocal off
        data[name] = np.frombuffer(b[off:off + 8 * n]).copy()
        off += 8 * n

    take("C066", 36); take("S066", 36); take("C_gr", 36 * N); take("Schm_xt", 120)
    take("Schm_gr", 60 * N); take("Chi", 144); take("Chi_1", 144); take("Shear_G", 2)
    take("bb_B", 24); take("TranMat", 9 * N); take("Sig", 9 * N); take("scalars", 4)
    take("S0", 81); take("B", 54)
    stride = 5
    for k in ("C_gr", "Schm_gr", "TranMat", "Sig"):
        w = data[k].size // N
        data[k] = data[k].reshape(N, w)[::stride]
    np.savez_compressed(out, spec=json.dumps(spec), stride=stride, **data)


def gen_nrprobe8(out: str) -> None:
    """One UpdateStress sweep on the bicrystal's initial state with a
    displacement gradient perturbed by a seeded random field."""
    spec = dict(kind="bicrystal8", steps=1, nr="plain")
    rng = np.random.default_rng(8)
    N = 512
    with tempfile.TemporaryDirectory() as t:
        case = make_input(spec, t)
        subprocess.run([REF, "input", "--setup", "setup.bin"], cwd=t, capture_output=True,
                       check=True)
        b = open(os.path.join(t, "setup.bin"), "rb").read()
        off = 8 + 8 * (36 + 36 + 36 * N + 120 + 60 * N + 144 + 144 + 2 + 24 + 9 * N)
        sig = np.frombuffer(b[off:off + 72 * N]).reshape(N, 9).copy()
        disgrad = np.zeros((N, 9))
        base = np.array([-0.5e-4, 0, 0, 0, 1.0e-4, 0, 0, 0, -0.5e-4])
        disgrad[:] = base + 3e-5 * rng.standard_normal((N, 9))
        eps = np.zeros((N, 9))
        rho_s = np.full((N, 12), 1.0) * (1.0 + 0.5 * rng.random((N, 12)))
        rho_m = 0.02 * rng.random((N, 12))
        inp = os.path.join(t, "probe_in.bin")
        with open(inp, "wb") as f:
            for a in (sig, disgrad, eps, rho_s, rho_m):
                f.write(np.ascontiguousarray(a).tobytes())
        subprocess.run([REF, "input", "--nr", "probe_in.bin", "probe_out.bin"], cwd=t,
                       capture_output=True, check=True)
        o = np.fromfile(os.path.join(t, "probe_out.bin"))
    p = 0
    res = {}
    for k, w in (("Sig", 9), ("Edot", 9), ("rho_m", 12), ("gamdot", 12), ("trial_gam_acum", 12),
                 ("rho_F", 12), ("rho_P", 12)):
        res[k] = o[p:p + w * N].reshape(N, w)
        p += w * N
    res["err"] = o[p:p + 2]
    np.savez_compressed(out, spec=json.dumps(spec), in_sig=sig, in_disgrad=disgrad, in_eps=eps,
                        in_rho_s=rho_s, in_rho_m=rho_m, **res)


GENS = {
    "bicrystal8": lambda o: gen_bicrystal8(o),
    "voronoi16_ls": lambda o: gen_voronoi(voronoi16_spec(), o),
    "cfg0_32_ls": lambda o: gen_voronoi(cfg0_32_spec(), o, stride=7),
    "gnd12_ls": lambda o: gen_voronoi(gnd12_spec(), o),
    "cfg0_32_run": lambda o: gen_run(cfg0_32_run_spec(), o),
    "cfg1_64_ls": lambda o: gen_run(cfg1_64_spec(), o),
    "cfg2_128_ls": lambda o: gen_run(cfg2_128_spec(), o),
    "setup16": lambda o: gen_setup16(o),
    "nrprobe8": lambda o: gen_nrprobe8(o),
}


def main(argv):
    if not all(os.path.exists(p) for p in (REF, REF_LS, REF_GND)):
        raise SystemExit("build the reference oracle first: make -C oracle ref")
    names = argv or list(GENS)
    for n in names:
        out = os.path.join(HERE, n + ".npz")
        GENS[n](out)
        print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main(sys.argv[1:])
