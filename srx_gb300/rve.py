"""Synthetic RVEs and the reference's input formats.

Writes the three files the reference reads, in its own formats:

* the namelist ``input`` (parsed by ``GetNameList``, io.c:96-164; key table
  io.c:25-94);
* the slip-system file ``.sx`` (parsed by ``PlasticInit``, init.c:52-231);
* the voxel microstructure text, one line ``phi1 Phi phi2 i j k grain phase``
  per voxel in degrees with i slowest (read by ``InitMicroStruct``,
  init.c:253-301).

RVEs are periodic Voronoi tessellations: seeds uniform in [0,1)^3, each voxel
centre ((i+1/2)/n) assigned to the nearest seed under the minimum-image
distance, ties to the lowest seed index. Each grain gets a Bunge orientation
uniform on SO(3): phi1 = 360 u1, Phi = acos(2 u2 - 1), phi2 = 360 u3.
Random numbers come from ``numpy.random.default_rng(seed)``.
"""
from __future__ import annotations

import dataclasses
import os
from typing import Optional, Sequence

import numpy as np

# FCC {111}<110> slip systems in the order of the reference's Cu_p.sx mode 1.
FCC_SLIP = (
    ((1, 1, -1), (0, 1, 1)), ((1, 1, -1), (1, 0, 1)), ((1, 1, -1), (1, -1, 0)),
    ((1, -1, -1), (0, 1, -1)), ((1, -1, -1), (1, 0, 1)), ((1, -1, -1), (1, 1, 0)),
    ((1, -1, 1), (0, 1, 1)), ((1, -1, 1), (1, 0, -1)), ((1, -1, 1), (1, 1, 0)),
    ((1, 1, 1), (0, 1, -1)), ((1, 1, 1), (1, 0, -1)), ((1, 1, 1), (1, -1, 0)),
)

# Load paths as (VelGrad_BC_Flag, VelGrad_BC direction, Stress_BC_Flag), Voigt
# order 11,22,33,23,13,12 (evolution.c:599). "shear" is the reference's
# symmetrised xy shear (kinematics.c:5-12).
LOADS = {
    "tension": ((0, 0, 1, 1, 1, 1), (0, 0, 1, 0, 0, 0), (1, 1, 0, 0, 0, 0)),
    "compression": ((0, 0, 1, 1, 1, 1), (0, 0, -1, 0, 0, 0), (1, 1, 0, 0, 0, 0)),
    "shear": ((0, 0, 0, 1, 1, 1), (0, 0, 0, 0, 0, 1), (1, 1, 1, 0, 0, 0)),
}


@dataclasses.dataclass
class Material:
    """Namelist material block; defaults are the FCC Cu set of the benchmark
    configurations (elastic constants in MPa, densities in 1e12 m^-2)."""

    c11: float = 168400.0
    c12: float = 121400.0
    c44: float = 75400.0
    nu: float = 0.35
    a0: float = 0.362
    T: float = 300.0
    q_slip: float = 2.0
    q_bulk: float = 1.6
    c1: float = 1.0
    c2: float = 1.0
    c3: float = 1.0
    c4: float = 600.0
    c5: float = 17.6
    c6: float = 0.0
    c7: float = 0.0
    c8: float = 0.24
    self_inter: float = 0.2
    coplanar: float = 0.2
    cross_slip: float = 0.2
    glissile: float = 0.3
    hirth: float = 0.2
    lomer: float = 0.4
    d0: float = 1.5e-3
    rho_ssd_initial: float = 1.0
    tau0: float = 0.0


@dataclasses.dataclass
class Job:
    """One run of the increment loop: grid, load path and controls."""

    n: Sequence[int]
    load: str = "tension"
    rate: float = 1e-3
    strain_per_step: float = 2e-4
    n_steps: int = 50
    err: float = 1e-5
    iter_max: int = 1000
    elast_bc: int = 1
    print_control: Sequence[int] = (0, 1)
    update_flag: int = 1
    hard_flag: int = 1
    # explicit load (overrides `load`/`rate`): Voigt flags and values
    velgrad_flag: Optional[Sequence[int]] = None
    velgrad: Optional[Sequence[float]] = None
    stress_flag: Optional[Sequence[int]] = None
    time_step_override: Optional[float] = None
    second_phase_gas: bool = False

    @property
    def time_step(self) -> float:
        if self.time_step_override is not None:
            return self.time_step_override
        return self.strain_per_step / self.rate


def voronoi(n: Sequence[int], n_grains: int, seed: int):
    """Periodic Voronoi grain ids (1-based, int32 [n0,n1,n2]) and per-grain
    Bunge angles in degrees ([n_grains,3])."""
    n = [int(x) for x in n]
    rng = np.random.default_rng(seed)
    seeds = rng.random((n_grains, 3))
    u = rng.random((n_grains, 3))
    euler = np.stack(
        [360.0 * u[:, 0], np.degrees(np.arccos(2.0 * u[:, 1] - 1.0)), 360.0 * u[:, 2]], axis=1
    )
    axes = [(np.arange(k) + 0.5) / k for k in n]
    if int(np.prod(n)) > 64 ** 3:
        # large grids: periodic k-d tree; exact distance ties are resolved to
        # the lower seed index as below
        from scipy.spatial import cKDTree
        pts = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).reshape(-1, 3)
        d, i = cKDTree(seeds, boxsize=1.0).query(pts, k=2, workers=-1)
        tie = d[:, 0] == d[:, 1]
        best = np.where(tie, np.minimum(i[:, 0], i[:, 1]), i[:, 0])
        return (best + 1).astype(np.int32).reshape(n), euler
    gid = np.zeros(n, dtype=np.int32)
    best = np.full(n, np.inf)
    cx, cy, cz = np.meshgrid(*axes, indexing="ij")
    for s in range(n_grains):
        d = 0.0
        for c, p in ((cx, seeds[s, 0]), (cy, seeds[s, 1]), (cz, seeds[s, 2])):
            t = np.abs(c - p)
            t = np.minimum(t, 1.0 - t)
            d = d + t * t
        take = d < best  # strict: ties stay with the lower seed index
        best = np.where(take, d, best)
        gid = np.where(take, s + 1, gid)
    return gid, euler


def write_microstructure(path: str, gid: np.ndarray, euler: np.ndarray,
                         phase: Optional[np.ndarray] = None) -> None:
    """Voxel text in the reference format (init.c:262), i slowest, 1-based."""
    n0, n1, n2 = gid.shape
    ang = euler[gid.reshape(-1) - 1]
    ii, jj, kk = np.meshgrid(np.arange(1, n0 + 1), np.arange(1, n1 + 1), np.arange(1, n2 + 1),
                             indexing="ij")
    ph = np.ones(gid.size, dtype=np.int64) if phase is None else phase.reshape(-1)
    rows = zip(ang[:, 0], ang[:, 1], ang[:, 2], ii.reshape(-1), jj.reshape(-1), kk.reshape(-1),
               gid.reshape(-1), ph)
    with open(path, "w") as f:
        f.write("".join("%.10f %.10f %.10f %d %d %d %d %d\n" % r for r in rows))


def write_sx(path: str, tau0: float = 0.0) -> None:
    """Slip-system file in the reference layout (init.c:52-160): one FCC
    {111}<110> mode with lattice resistance tau0xf = tau0."""
    lines = [
        "# Crystal system (XtalSys):", "CUBIC", "", "# Crystal axex (XtalAxis):", "1.0 1.0 1.0",
        "", "# Total number of modes listed in the file (N_modes_max):", "1", "",
        "# Number of modes to be used in the calculation (N_modes):", "1", "",
        "# Labels of the modes to be used (iMode):", "1", "",
        "# Mode# 1 -- <110>(111) SLIP",
        "\tnsmx\tnrsx\tgamd0x\ttwshx\tisectwx", "\t12\t\t10.\t\t1.0\t\t0.0\t\t0",
        "\ttau0xf\ttau0xb\ttau1x\tthet0\tthet1",
        "\t%r\t\t%r\t\t5.\t\t400.\t\t250." % (float(tau0), float(tau0)),
        "\thselfx\thlatex", "\t1.0\t\t1.0", "\tSlip (n-b)",
    ]
    for nvec, bvec in FCC_SLIP:
        lines.append("\t%d %d %d\t\t%d %d %d" % (*nvec, *bvec))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_namelist(path: str, job: Job, mat: Material, ms_name: str, sx_name: str) -> None:
    """Namelist in the reference format (key table io.c:25-94)."""
    flag_v, direction, flag_s = LOADS[job.load]
    vel = [d * job.rate for d in direction]
    if job.velgrad_flag is not None:
        flag_v, vel, flag_s = job.velgrad_flag, list(job.velgrad), job.stress_flag
    n = [int(x) for x in job.n]
    m = mat
    kv = [
        ("N_phases", "2"), ("CellDim", "%d %d %d" % tuple(n)), ("initial_ms", ms_name),
        ("Type_phases", "0 1" if job.second_phase_gas else "0 0"),
        ("ElastConst_PhaseI", "%r %r %r %r" % (m.c11, m.c12, m.c44, m.nu)),
        ("Slip_PhaseI", sx_name),
        ("ElastConst_PhaseII", "%r %r %r %r" % (m.c11, m.c12, m.c44, m.nu)),
        ("Slip_PhaseII", sx_name),
        ("VelGrad_BC_Flag", " ".join(str(x) for x in flag_v)),
        ("VelGrad_BC", " ".join(repr(float(x)) for x in vel)),
        ("Stress_BC_Flag", " ".join(str(x) for x in flag_s)),
        ("Stress_BC", "0. 0. 0. 0. 0. 0."), ("ElastBC", str(job.elast_bc)),
        ("TimeStep", repr(float(job.time_step))), ("N_steps", str(job.n_steps)),
        ("Err", repr(float(job.err))), ("IterMax", str(job.iter_max)),
        ("PrintControl", "%d %d" % tuple(job.print_control)),
        ("Update_Flag", str(job.update_flag)), ("Hard_Flag", str(job.hard_flag)),
        ("Tex_Flag", "1"), ("a0", "%r %r" % (m.a0, m.a0)), ("L0", "0.0045"),
        ("GND_ScaleRatio", "200.0"), ("Q_slip", "%r %r" % (m.q_slip, m.q_slip)),
        ("Q_bulk", "%r %r" % (m.q_bulk, m.q_bulk)), ("rho_SSD_initial", repr(m.rho_ssd_initial)),
        ("T__K", repr(m.T)), ("C_1", "%r %r" % (m.c1, m.c1)), ("C_2", "%r %r" % (m.c2, m.c2)),
        ("C_3", "%r %r" % (m.c3, m.c3)), ("C_4", "%r %r" % (m.c4, m.c4)),
        ("C_5", "%r %r" % (m.c5, m.c5)), ("C_6", "%r %r" % (m.c6, m.c6)),
        ("C_7", "%r %r" % (m.c7, m.c7)), ("C_8", "%r %r" % (m.c8, m.c8)),
        ("Selfinter0", "%r %r" % (m.self_inter, m.self_inter)),
        ("Coplanar0", "%r %r" % (m.coplanar, m.coplanar)),
        ("CrossSlip0", "%r %r" % (m.cross_slip, m.cross_slip)),
        ("GlissileJunction0", "%r %r" % (m.glissile, m.glissile)),
        ("HirthLock0", "%r %r" % (m.hirth, m.hirth)),
        ("LomerCottrellLock0", "%r %r" % (m.lomer, m.lomer)), ("D_0", repr(m.d0)),
        ("nucleus_radius", "4"), ("CellDim_pf", "%d %d %d" % tuple(n)), ("RandSeed", "123"),
        ("E_gb", "0.625"), ("M_gb", "7.4E-11"), ("Scale_Fdeform", "0.5"), ("k_c", "320000.0"),
        ("alpha", "8.5"), ("zeta_kc", "1.0"), ("age_drx", "1E0"), ("ssdScaler_DRX", "0.74"),
        ("gndScaler_DRX", "0.66"), ("sigScaler_DRX", "0.66"), ("Nucl_Static_Flag", "1"),
        ("tau_DRX", "1000.0"), ("DeltaQ_DRX", "0.0"), ("DeltaTau_DRX", "0.0"),
        ("pf_length_scale", "2.5E-06"), ("pf_time_step", "0.004"),
    ]
    with open(path, "w") as f:
        f.write("# EVP-FFT namelist\n")
        for k, v in kv:
            f.write("%s\t%s\n" % (k, v))


def per_grain_rho0(gid: np.ndarray, lo: float, hi: float, seed: int) -> np.ndarray:
    """Per-voxel initial SSD density (1e12 m^-2), log-uniform in [lo, hi] per
    grain; float64 in voxel order."""
    rng = np.random.default_rng(seed)
    g = int(gid.max())
    vals = np.exp(rng.uniform(np.log(lo), np.log(hi), size=g))
    return vals[gid.reshape(-1) - 1].astype(np.float64)


def make_case(dirpath: str, n: Sequence[int], n_grains: int, seed: int, job: Job,
              mat: Optional[Material] = None, rho0: Optional[Sequence[float]] = None,
              euler: Optional[np.ndarray] = None) -> dict:
    """Write a complete case directory (input, cu.sx, ms.txt[, rho0.bin]) and
    return its paths. ``rho0=(lo, hi)`` adds a per-grain log-uniform initial
    density file; ``euler`` overrides the random grain orientations."""
    mat = mat or Material()
    os.makedirs(dirpath, exist_ok=True)
    gid, eul = voronoi(n, n_grains, seed)
    if euler is not None:
        eul = np.asarray(euler, dtype=np.float64).reshape(-1, 3)
    write_microstructure(os.path.join(dirpath, "ms.txt"), gid, eul)
    write_sx(os.path.join(dirpath, "cu.sx"), mat.tau0)
    job = dataclasses.replace(job, n=tuple(int(x) for x in n))
    write_namelist(os.path.join(dirpath, "input"), job, mat, "ms.txt", "cu.sx")
    out = {"dir": dirpath, "input": os.path.join(dirpath, "input"), "rho0": None,
           "gid": gid, "euler": eul}
    if rho0 is not None:
        r = per_grain_rho0(gid, rho0[0], rho0[1], seed + 7919)
        p = os.path.join(dirpath, "rho0.bin")
        r.tofile(p)
        out["rho0"] = p
    return out


def write_case(dirpath: str, gid: np.ndarray, euler: np.ndarray, job: Job,
               mat: Optional[Material] = None, phase: Optional[np.ndarray] = None,
               rho0: Optional[np.ndarray] = None) -> dict:
    """Case directory for an explicit grain map ``gid`` (1-based [n0,n1,n2]),
    per-grain Bunge angles ``euler`` in degrees and optional per-voxel phase
    ids and initial densities."""
    mat = mat or Material()
    os.makedirs(dirpath, exist_ok=True)
    write_microstructure(os.path.join(dirpath, "ms.txt"), gid, np.asarray(euler, float), phase)
    write_sx(os.path.join(dirpath, "cu.sx"), mat.tau0)
    job = dataclasses.replace(job, n=tuple(int(x) for x in gid.shape))
    write_namelist(os.path.join(dirpath, "input"), job, mat, "ms.txt", "cu.sx")
    out = {"dir": dirpath, "input": os.path.join(dirpath, "input"), "rho0": None}
    if rho0 is not None:
        p = os.path.join(dirpath, "rho0.bin")
        np.asarray(rho0, dtype=np.float64).reshape(-1).tofile(p)
        out["rho0"] = p
    return out


def bicrystal8_case(dirpath: str, n_steps: int = 5, print_every: int = 1) -> dict:
    """The reference's own 8^3 regression case, restated: planes i=1..4 with
    Bunge (0,0,0), planes i=5..8 with (90,35,45), one grain id, phase 1; Cu
    at c11/c12/c44 = 162700/119000/71150 MPa, tau0xf 0, interaction
    coefficients 0.1/0.125/0.125/0.15/0.1/0.2; mixed-BC y tension
    (VelGrad_BC -0.5e-3 1e-3 -0.5e-3, xx and zz stress free), TimeStep 0.1,
    Err 5e-5, second phase gas, plain NR."""
    gid = np.ones((8, 8, 8), dtype=np.int32)
    gid[4:] = 2  # two orientation rows; the grain id written stays 1 below
    euler = np.array([[0.0, 0.0, 0.0], [90.0, 35.0, 45.0]])
    mat = Material(c11=162700.0, c12=119000.0, c44=71150.0, nu=0.35, tau0=0.0,
                   self_inter=0.1, coplanar=0.125, cross_slip=0.125, glissile=0.15,
                   hirth=0.1, lomer=0.2, rho_ssd_initial=1.0)
    job = Job(n=(8, 8, 8), n_steps=n_steps, err=5e-5, iter_max=1000,
              print_control=(1, print_every), velgrad_flag=(0, 1, 0, 1, 1, 1),
              velgrad=(-0.5e-3, 1.0e-3, -0.5e-3, 0.0, 0.0, 0.0),
              stress_flag=(1, 0, 1, 0, 0, 0), time_step_override=0.1, second_phase_gas=True)
    os.makedirs(dirpath, exist_ok=True)
    ang = euler[gid.reshape(-1) - 1]
    with open(os.path.join(dirpath, "ms.txt"), "w") as f:
        for v in range(512):
            i, j, k = v // 64 + 1, (v // 8) % 8 + 1, v % 8 + 1
            f.write("%g %g %g %d %d %d 1 1\n" % (ang[v, 0], ang[v, 1], ang[v, 2], i, j, k))
    write_sx(os.path.join(dirpath, "cu.sx"), mat.tau0)
    write_namelist(os.path.join(dirpath, "input"), job, mat, "ms.txt", "cu.sx")
    return {"dir": dirpath, "input": os.path.join(dirpath, "input"), "rho0": None}


def main(argv=None) -> None:
    """Write one seeded synthetic case directory:

        python -m srx_gb300.rve --out DIR --n 64 --grains 125 [--seed S]
            [--load tension|compression|shear] [--rate R] [--steps K]
            [--rho0 LO HI]
    """
    import argparse
    p = argparse.ArgumentParser(prog="python -m srx_gb300.rve")
    p.add_argument("--out", required=True)
    p.add_argument("--n", type=int, nargs="+", default=[32])
    p.add_argument("--grains", type=int, default=27)
    p.add_argument("--seed", type=int, default=2025)
    p.add_argument("--load", default="tension", choices=["tension", "compression", "shear"])
    p.add_argument("--rate", type=float, default=1e-3)
    p.add_argument("--strain-per-step", type=float, default=2e-4)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--err", type=float, default=1e-5)
    p.add_argument("--rho0", type=float, nargs=2, default=None)
    a = p.parse_args(argv)
    n = tuple(a.n * 3 if len(a.n) == 1 else a.n)
    job = Job(n=n, load=a.load, rate=a.rate, strain_per_step=a.strain_per_step,
              n_steps=a.steps, err=a.err)
    c = make_case(a.out, n, a.grains, a.seed, job, rho0=a.rho0)
    print(c["input"], c["rho0"] or "")


if __name__ == "__main__":
    main()
