"""Seeded synthetic workloads of the batching and serving forms.

Batching: independent RVEs of uneven grids (n^3, n in {16, 32, 48, 64}),
8-200 Voronoi grains with uniform-random orientations, a load drawn from
{z tension, z compression, xy shear} and a strain rate log-uniform in
[1e-4, 1e-2]/s.

Serving: a stream of solve requests, grid n^3 with n in {32, 64, 96, 128},
8-1000 grains, a load path from {tension, compression, shear,
tension-then-shear}, strain rate log-uniform in [1e-4, 1e-2]/s and Poisson
arrival times.

Increments are 2e-4 strain for tension and compression and 1e-4 for shear
(the reference's Newton-Raphson fails on xy shear at 2e-4 per increment with
this material); a tension-then-shear request runs both legs at 1e-4 with
the switch half way.
"""
from __future__ import annotations

import os
from typing import List

import numpy as np

from . import rve

STRAIN_STEP = {"tension": 2e-4, "compression": 2e-4, "shear": 1e-4}


def _case(d: str, n: int, grains: int, load: str, rate: float, steps: int, seed: int) -> dict:
    sps = STRAIN_STEP.get(load, 1e-4)
    first = "tension" if load == "tension-then-shear" else load
    job = rve.Job(n=(n,) * 3, load=first, rate=rate, strain_per_step=sps, n_steps=steps)
    c = rve.make_case(d, (n,) * 3, grains, seed, job, rho0=(0.5, 5.0))
    c.update({"n": n, "grains": grains, "load": load, "rate": rate, "steps": steps,
              "N": n ** 3, "switch": -1, "switch_input": None})
    if load == "tension-then-shear":
        shear = rve.Job(n=(n,) * 3, load="shear", rate=rate, strain_per_step=sps, n_steps=steps)
        p = os.path.join(d, "input_shear")
        rve.write_namelist(p, shear, rve.Material(), "ms.txt", "cu.sx")
        c["switch"] = max(1, steps // 2)
        c["switch_input"] = p
    return c


def batch_set(root: str, count: int = 64, steps: int = 100, seed: int = 3000,
              sizes=(16, 32, 48, 64)) -> List[dict]:
    """`count` RVE cases of the batching form under `root`."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.choice(sizes))
        grains = int(rng.integers(8, 201))
        load = str(rng.choice(["tension", "compression", "shear"]))
        rate = float(10 ** rng.uniform(-4, -2))
        out.append(_case(os.path.join(root, "b%03d" % i), n, grains, load, rate, steps, seed + 1 + i))
    return out


def serve_stream(root: str, count: int, rate_hz: float, steps=(20, 200), seed: int = 4000,
                 sizes=(32, 64, 96, 128), distinct: int = 0) -> List[dict]:
    """`count` requests with Poisson arrival offsets `t` (seconds) at
    `rate_hz`. With distinct > 0 only that many case directories are written
    and requests cycle through them (each request still opens its own copy
    of the RVE on the device)."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_hz, size=count))
    arrivals -= arrivals[0]
    ncase = distinct if distinct > 0 else count
    cases = []
    for i in range(ncase):
        n = int(rng.choice(sizes))
        grains = int(rng.integers(8, 1001))
        load = str(rng.choice(["tension", "compression", "shear", "tension-then-shear"]))
        rate = float(10 ** rng.uniform(-4, -2))
        k = int(rng.integers(steps[0], steps[1] + 1))
        cases.append(_case(os.path.join(root, "s%03d" % i), n, grains, load, rate, k, seed + 1 + i))
    return [dict(cases[i % ncase], t=float(arrivals[i])) for i in range(count)]
