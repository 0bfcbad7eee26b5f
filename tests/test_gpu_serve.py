"""Continuous-batching server (evpg_server_*): every request's result is the
same alone and in the mix -- bit-identical stress, SSD density and scalars
-- while requests of different grids, loads and lengths arrive during
others' work, wait for slots, and (with a small device-memory budget) wait
for memory. Includes a tension-then-shear request (mid-run load switch)."""
import os
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _evpg():
    from srx_gb300 import build, evpg
    build.build()
    return evpg


def _requests(tmp_path):
    from srx_gb300 import rve
    specs = [  # grid, grains, load, rate, strain/increment, increments, switch step
        ((16, 16, 16), 8, "tension", 1e-3, 2e-4, 3, -1),
        ((12, 10, 9), 6, "compression", 3e-3, 2e-4, 2, -1),
        ((16, 12, 8), 10, "tension", 1e-3, 1e-4, 4, 2),   # then shear
        ((20, 16, 12), 5, "shear", 5e-4, 1e-4, 2, -1),
        ((8, 8, 8), 3, "tension", 2e-3, 2e-4, 3, -1),
    ]
    out = []
    for i, (n, grains, load, rate, sps, steps, sw) in enumerate(specs):
        d = str(tmp_path / ("r%d" % i))
        job = rve.Job(n=n, load=load, rate=rate, strain_per_step=sps, n_steps=steps)
        c = rve.make_case(d, n, grains, 100 + i, job, rho0=(0.5, 5.0))
        c["steps"], c["switch"], c["N"] = steps, sw, int(np.prod(n))
        c["switch_input"] = None
        if sw > 0:
            shear = rve.Job(n=n, load="shear", rate=rate, strain_per_step=sps, n_steps=steps)
            p = os.path.join(d, "input_shear")
            rve.write_namelist(p, shear, rve.Material(), "ms.txt", "cu.sx")
            c["switch_input"] = p
        out.append(c)
    return out


def _alone(evpg, c, precision):
    with evpg.Job(c["input"], c["rho0"], precision=precision, nr_mode=1) as j:
        for k in range(c["steps"]):
            if c["switch"] > 0 and k == c["switch"]:
                j.set_load_from(c["switch_input"])
            j.increment(k)
        return j.download(evpg.F_SIG6), j.download(evpg.F_RHO_S), j.scalars()


@pytest.mark.parametrize("precision", [0, 1])
def test_served_results_equal_alone(tmp_path, precision):
    evpg = _evpg()
    reqs = _requests(tmp_path)
    ref = [_alone(evpg, c, precision) for c in reqs]
    with evpg.Server(precision=precision, nr_mode=1, max_slots=3, round_ticks=13, loaders=2,
                     keep_fields=True) as srv:
        ids = []
        for c in reqs:
            ids.append(srv.submit(c["input"], c["steps"], rho0=c["rho0"], switch_step=c["switch"],
                                  switch_input=c["switch_input"]))
            time.sleep(0.02)
        srv.wait(600)
        st = srv.stats()
        assert st.completed == len(reqs) and st.failed == 0
        assert st.increments == sum(c["steps"] for c in reqs)
        assert 0 < st.incr_p50 <= st.incr_p99 and 0 < st.solve_p50 <= st.solve_p99
        assert st.solves_per_s > 0
        for rid, c, (sig, rho, sc) in zip(ids, reqs, ref):
            info = srv.request(rid)
            assert info.state == 4 and info.increments == c["steps"]
            gs, gr, gsc = srv.result(rid, c["N"])
            assert np.array_equal(gs, sig)
            assert np.array_equal(gr, rho)
            assert np.array_equal(gsc, sc)


def test_admission_by_memory_budget(tmp_path):
    """With room for one request at a time (reservations 26, 19 and 20 MB in a
    30 MB budget), solves run one after another."""
    evpg = _evpg()
    reqs = _requests(tmp_path)[:3]
    with evpg.Server(precision=1, nr_mode=1, hbm_budget=30 << 20, max_slots=8, round_ticks=16,
                     loaders=3) as srv:
        ids = [srv.submit(c["input"], c["steps"], rho0=c["rho0"], switch_step=c["switch"],
                          switch_input=c["switch_input"]) for c in reqs]
        srv.wait(600)
        iv = sorted((srv.request(i).t_admit, srv.request(i).t_done) for i in ids)
        assert all(srv.request(i).state == 4 for i in ids)
        for (a0, d0), (a1, d1) in zip(iv, iv[1:]):
            assert d0 <= a1


def test_request_larger_than_budget_fails(tmp_path):
    evpg = _evpg()
    c = _requests(tmp_path)[0]
    with evpg.Server(precision=1, nr_mode=1, hbm_budget=1 << 20, max_slots=4, round_ticks=16) as srv:
        rid = srv.submit(c["input"], 1, rho0=c["rho0"])
        srv.wait(60)
        info = srv.request(rid)
        assert info.state == 5 and info.status == 3  # EVPG_ERR_NOMEM


def test_failing_request_fails_alone(tmp_path):
    """xy shear at 2e-4 per increment makes the Newton-Raphson fail in its
    first iteration (the reference's own NR fails there too). In the server
    that request ends with its error status; the requests around it finish
    with the same results as alone."""
    from srx_gb300 import rve
    evpg = _evpg()
    good = _requests(tmp_path)[:2]
    n = (16, 16, 16)
    job = rve.Job(n=n, load="shear", rate=1e-3, strain_per_step=2e-4, n_steps=2)
    bad = rve.make_case(str(tmp_path / "bad"), n, 8, 7, job, rho0=(0.5, 5.0))
    with evpg.Job(bad["input"], bad["rho0"], precision=1, nr_mode=1) as j:
        with pytest.raises(evpg.EvpgError) as ei:
            j.increment(0)
        assert ei.value.status in (4, 5, 6)  # NaN, singular, line search
    ref = [_alone(evpg, c, 1) for c in good]
    with evpg.Server(precision=1, nr_mode=1, max_slots=4, round_ticks=11, keep_fields=True) as srv:
        ids = [srv.submit(good[0]["input"], good[0]["steps"], rho0=good[0]["rho0"]),
               srv.submit(bad["input"], 2, rho0=bad["rho0"]),
               srv.submit(good[1]["input"], good[1]["steps"], rho0=good[1]["rho0"])]
        srv.wait(600)
        info = srv.request(ids[1])
        assert info.state == 5 and info.status in (4, 5, 6)
        for rid, c, (sig, rho, sc) in zip((ids[0], ids[2]), good, ref):
            assert srv.request(rid).state == 4
            gs, gr, gsc = srv.result(rid, c["N"])
            assert np.array_equal(gs, sig) and np.array_equal(gr, rho) and np.array_equal(gsc, sc)


def test_served_gnd_requests_equal_alone(tmp_path):
    """A server opened with GND densities (job option of every request):
    four-increment solves in the mix give the same bits as each alone."""
    from srx_gb300 import rve
    evpg = _evpg()
    reqs = []
    for i, (n, load) in enumerate((((12, 12, 12), "tension"), ((16, 12, 8), "compression"))):
        job = rve.Job(n=n, load=load, rate=1e-3, strain_per_step=2e-4, n_steps=4)
        c = rve.make_case(str(tmp_path / ("g%d" % i)), n, 5, 300 + i, job, rho0=(0.5, 5.0))
        c["N"] = int(np.prod(n))
        reqs.append(c)
    ref = []
    for c in reqs:
        with evpg.Job(c["input"], c["rho0"], precision=1, nr_mode=1, gnd=True) as j:
            for k in range(4):
                j.increment(k)
            ref.append((j.download(evpg.F_SIG6), j.download(evpg.F_RHO_S), j.scalars()))
    with evpg.Server(precision=1, nr_mode=1, max_slots=2, round_ticks=17, keep_fields=True,
                     gnd=True) as srv:
        ids = [srv.submit(c["input"], 4, rho0=c["rho0"]) for c in reqs]
        srv.wait(600)
        for rid, c, (sig, rho, sc) in zip(ids, reqs, ref):
            assert srv.request(rid).state == 4
            gs, gr, gsc = srv.result(rid, c["N"])
            assert np.array_equal(gs, sig) and np.array_equal(gr, rho) and np.array_equal(gsc, sc)
