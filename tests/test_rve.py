"""Synthetic RVE generator and the reference input formats."""
import numpy as np

from srx_gb300 import rve


def test_voronoi_is_periodic_nearest_seed_with_low_index_ties():
    n = (6, 5, 4)
    gid, euler = rve.voronoi(n, 5, seed=3)
    rng = np.random.default_rng(3)
    seeds = rng.random((5, 3))
    for i in range(n[0]):
        for j in range(n[1]):
            for k in range(n[2]):
                c = (np.array([i, j, k]) + 0.5) / np.array(n)
                d = np.abs(seeds - c)
                d = np.minimum(d, 1 - d)
                dist = (d * d).sum(1)
                assert gid[i, j, k] == int(np.argmin(dist)) + 1
    assert euler.shape == (5, 3)
    assert np.all((euler[:, 1] >= 0) & (euler[:, 1] <= 180))


def test_orientations_uniform_on_so3():
    _, e = rve.voronoi((2, 2, 2), 20000, seed=1)
    # cos(Phi) uniform on [-1,1] for the Haar measure in Bunge angles
    c = np.cos(np.radians(e[:, 1]))
    assert abs(c.mean()) < 0.02 and abs(np.var(c) - 1 / 3) < 0.01


def test_case_files_parse_in_the_oracle(oracle, tmp_path):
    case = rve.make_case(str(tmp_path / "c"), (6, 4, 5), 4, 2, rve.Job(n=(6, 4, 5), n_steps=7),
                         rho0=(0.5, 5.0))
    h = oracle.open(case["input"], case["rho0"])
    try:
        assert oracle.L.evo_nvox(h) == 120
        rho = oracle.field(h, "rho_s", 120 * 12).reshape(120, 12)
        r0 = np.fromfile(case["rho0"])
        assert np.array_equal(rho[:, 0], r0) and np.all((r0 >= 0.5) & (r0 <= 5.0))
    finally:
        oracle.L.evo_close(h)
