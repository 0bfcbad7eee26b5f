"""Batched RVEs (one launch per kernel over all RVEs, one CUDA graph per
round) against the same RVEs run alone through the C ABI.

Every RVE of a batch runs the same per-RVE arithmetic as alone (same pencil
schedules, deterministic reductions), so the results must be bit-identical:
iteration counts per increment and every state field. Uneven grids
(including odd and mixed-radix lengths), loads and strain rates are mixed,
and rounds are cut short (max_ticks) so RVEs finish their increments in
different rounds and start the next one while others are still iterating.
Shear increments are 1e-4 (the reference's NR fails on xy shear at 2e-4 per
increment with this material)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = None


def _evpg():
    from srx_gb300 import build, evpg
    build.build()
    return evpg


def _cases(tmp_path):
    from srx_gb300 import rve
    specs = [
        ((16, 16, 16), 8, "tension", 1e-3, 2e-4, 11),
        ((12, 10, 9), 6, "compression", 3e-3, 2e-4, 12),
        ((16, 12, 8), 10, "shear", 1e-3, 1e-4, 13),
        ((20, 16, 12), 5, "tension", 5e-4, 2e-4, 14),
        ((8, 8, 8), 3, "shear", 2e-3, 1e-4, 15),
    ]
    out = []
    for i, (n, grains, load, rate, sps, seed) in enumerate(specs):
        job = rve.Job(n=n, load=load, rate=rate, strain_per_step=sps, n_steps=4)
        out.append(rve.make_case(str(tmp_path / ("c%d" % i)), n, grains, seed, job, rho0=(0.5, 5.0)))
    return out


def _state(evpg, j):
    return {f: j.download(f) for f in (evpg.F_SIG6, evpg.F_DISGRAD, evpg.F_RHO_S, evpg.F_EPS,
                                       evpg.F_TRANMAT, evpg.F_GAM_ACUM)}


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_equals_alone(tmp_path, precision):
    evpg = _evpg()
    cases = _cases(tmp_path)
    nsteps = [3, 2, 3, 1, 3]
    alone_it, alone_st, alone_sc = [], [], []
    for c, ns in zip(cases, nsteps):
        with evpg.Job(c["input"], c["rho0"], precision=precision, nr_mode=1) as j:
            alone_it.append([j.increment(k) for k in range(ns)])
            alone_st.append(_state(evpg, j))
            alone_sc.append(j.scalars())
    jobs = [evpg.Job(c["input"], c["rho0"], precision=precision, nr_mode=1) for c in cases]
    try:
        its, rounds = evpg.run_batched(jobs, nsteps, max_ticks=23)
        assert its == alone_it
        assert rounds > max(sum(x) for x in alone_it) // 23  # rounds were cut short
        for j, st, sc in zip(jobs, alone_st, alone_sc):
            got = _state(evpg, j)
            for f, v in st.items():
                assert np.array_equal(got[f], v), f
            assert np.array_equal(j.scalars(), sc)
    finally:
        for j in jobs:
            j.close()


def test_graph_increment_launch_count(tmp_path):
    """One increment through the round graph launches prologue + ticks x body
    kernels + the increment tail once (a conditional node that runs only in
    the iteration where the loop ends); the context's counter reflects the
    kernels that ran."""
    evpg = _evpg()
    c = _cases(tmp_path)[0]
    with evpg.Job(c["input"], c["rho0"], precision=1, nr_mode=1) as j:
        fused = j.variant()[0] > 0
        # with both warp-register passes the deferred antisymmetric part adds
        # its X pass flush and inverse plane pass to the tail
        flush = 2 if fused and j.variant()[1] > 0 else 0
        n0 = j.launches()
        it = j.increment(0)
        n1 = j.launches()
    # prologue: macro reset, head, round start and the first iteration's
    # forward transforms with the X pass (2 with the fused plane kernels, else
    # 3); body: inverse transforms, NR, macro update, the next iteration's
    # forward transforms, tail test, advance = 9 per iteration with the
    # separate passes (7 fused); tail: fold + FP64 refinement + tail 2 = 4, once
    fwd = 2 if fused else 3
    body = (3 if fused else 5) + 4
    assert n1 - n0 == 3 + fwd + body * it + 4 + flush


def test_batch_rejects_mixed_precision(tmp_path):
    import ctypes as C
    evpg = _evpg()
    c = _cases(tmp_path)[4]
    a = evpg.Job(c["input"], c["rho0"], precision=0, nr_mode=1)
    b = evpg.Job(c["input"], c["rho0"], precision=1, nr_mode=1)
    try:
        L = evpg.lib()
        h = C.c_void_p()
        evpg.check(L.evpg_batch_create(0, 1, C.byref(h)))
        ctxs = (C.c_void_p * 2)(a.ctx.value, b.ctx.value)
        assert L.evpg_batch_set(h, ctxs, 2) == 1
        L.evpg_batch_destroy(h)
    finally:
        a.close()
        b.close()


def test_autotuned_schedule(tmp_path):
    """The tuned schedule (radix orders, pencils per CTA) gives the same
    iterations and fields within FFT rounding (FP64), and a second context of
    the same grid takes it from the cache."""
    from conftest import rel_err
    evpg = _evpg()
    c = _cases(tmp_path)[1]  # 12 x 10 x 9: radix 4/2/3/5 and odd lengths
    res = []
    for tune in (False, True):
        with evpg.Job(c["input"], c["rho0"], precision=0, nr_mode=1) as j:
            if tune:
                g = j.tune(force=True)
                assert g > 0
                sched = j.schedule()
                assert [int(np.prod(r)) for r in sched["radix_xyz"]] == [12, 10, 9]
            its = [j.increment(k) for k in range(2)]
            res.append((its, j.download(evpg.F_SIG6), j.download(evpg.F_RHO_S)))
    assert res[0][0] == res[1][0]
    assert rel_err(res[1][1], res[0][1]) < 1e-9
    assert rel_err(res[1][2], res[0][2]) < 1e-9
    with evpg.Job(c["input"], c["rho0"], precision=0, nr_mode=1) as j:
        assert j.tune() == 0.0  # cached
        assert j.schedule() == sched


@pytest.mark.parametrize("grid,prec", [((16, 32, 32), 0), ((8, 64, 64), 0), ((8, 64, 64), 1),
                                       ((4, 128, 128), 1)])
def test_fused_plane_passes(tmp_path, grid, prec):
    """The fused z+y plane kernels (warp-register FFTs) against the separate
    Stockham passes on grids n1 == n2 = 32, 64, 128: FP64 within FFT rounding
    with the same iterations; FP32 bulk within its tolerance."""
    from conftest import rel_err
    from srx_gb300 import rve
    evpg = _evpg()
    job = rve.Job(n=grid, load="tension", rate=1e-3, strain_per_step=2e-4, n_steps=2)
    c = rve.make_case(str(tmp_path / "c"), grid, 6, 21, job, rho0=(0.5, 5.0))
    res = []
    for fused in (0, 1):
        with evpg.Job(c["input"], c["rho0"], precision=prec, nr_mode=1) as j:
            j.set_fused(fused)
            assert (j.schedule()["pencils_zyx"][0] == 0) == bool(fused)
            its = [j.increment(k) for k in range(2)]
            res.append((its, j.download(evpg.F_SIG6), j.download(evpg.F_RHO_S), j.scalars()))
    if prec == 0:
        assert res[0][0] == res[1][0]
        assert rel_err(res[1][1], res[0][1]) < 1e-9
        assert rel_err(res[1][2], res[0][2]) < 1e-9
    else:
        assert abs(sum(res[0][0]) - sum(res[1][0])) <= 2
        assert rel_err(res[1][3][7:16], res[0][3][7:16]) < 1e-5
        l2 = np.linalg.norm(res[1][1] - res[0][1]) / np.linalg.norm(res[0][1])
        assert l2 < 1e-4, l2


def test_batch_with_fused_planes_equals_alone(tmp_path):
    """Batched fused z+y kernels (every slot n1 == n2 == 32, FP32 bulk) give
    the same bits as each RVE alone."""
    from srx_gb300 import rve
    evpg = _evpg()
    cases = []
    for i, (grid, load, sps) in enumerate((((8, 32, 32), "tension", 2e-4), ((16, 32, 32), "shear", 1e-4),
                                           ((4, 32, 32), "compression", 2e-4), ((32, 32, 32), "shear", 1e-4))):
        job = rve.Job(n=grid, load=load, rate=1e-3, strain_per_step=sps, n_steps=2)
        cases.append(rve.make_case(str(tmp_path / ("f%d" % i)), grid, 5, 40 + i, job, rho0=(0.5, 5.0)))
    ref = []
    for c in cases:
        with evpg.Job(c["input"], c["rho0"], precision=1, nr_mode=1) as j:
            assert j.schedule()["pencils_zyx"][0] == 0  # fused by default
            ref.append(([j.increment(k) for k in range(2)], _state(evpg, j)))
    jobs = [evpg.Job(c["input"], c["rho0"], precision=1, nr_mode=1) for c in cases]
    try:
        # the 32^3 slot also runs the warp-register X pass: its antisymmetric
        # correction is deferred to the end of each increment
        assert [j.variant()[1] > 0 for j in jobs] == [False, False, False, True]
        its, _ = evpg.run_batched(jobs, [2, 2, 2, 2], max_ticks=19)
        assert its == [r[0] for r in ref]
        for j, (_, st) in zip(jobs, ref):
            got = _state(evpg, j)
            for f, v in st.items():
                assert np.array_equal(got[f], v), f
    finally:
        for j in jobs:
            j.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_mixing_fused_and_separate_passes(tmp_path, precision):
    """Slots with fused plane kernels of two lane layouts (32 and 64 planes)
    next to slots with the separate passes: each runs its own variant, so the
    batch gives the same bits as every RVE alone. FP64 contexts are switched
    to the fused kernels where eligible."""
    from srx_gb300 import rve
    evpg = _evpg()
    cases = []
    for i, (grid, load, sps) in enumerate((((8, 32, 32), "tension", 2e-4), ((4, 64, 64), "shear", 1e-4),
                                           ((12, 10, 9), "compression", 2e-4), ((16, 16, 16), "tension", 2e-4))):
        job = rve.Job(n=grid, load=load, rate=1e-3, strain_per_step=sps, n_steps=2)
        cases.append(rve.make_case(str(tmp_path / ("m%d" % i)), grid, 5, 60 + i, job, rho0=(0.5, 5.0)))

    def open_job(c):
        j = evpg.Job(c["input"], c["rho0"], precision=precision, nr_mode=1)
        j.set_fused(1)
        return j
    ref = []
    for c in cases:
        with open_job(c) as j:
            ref.append(([j.increment(k) for k in range(2)], _state(evpg, j)))
    jobs = [open_job(c) for c in cases]
    try:
        assert [j.schedule()["pencils_zyx"][0] == 0 for j in jobs] == [True, True, False, False]
        its, _ = evpg.run_batched(jobs, [2] * len(jobs), max_ticks=17)
        assert its == [r[0] for r in ref]
        for j, (_, st) in zip(jobs, ref):
            got = _state(evpg, j)
            for f, v in st.items():
                assert np.array_equal(got[f], v), f
    finally:
        for j in jobs:
            j.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_with_gnd_slot_equals_alone(tmp_path, precision):
    """A context with GND densities next to contexts without them in one
    batch: every RVE, the GND densities included, keeps its solo bits."""
    from srx_gb300 import rve
    evpg = _evpg()
    cases = []
    for i, (grid, load, gnd) in enumerate((((12, 12, 12), "tension", True), ((12, 10, 9), "compression", False),
                                           ((8, 8, 8), "tension", True))):
        job = rve.Job(n=grid, load=load, rate=1e-3, strain_per_step=2e-4, n_steps=4)
        c = rve.make_case(str(tmp_path / ("g%d" % i)), grid, 5, 80 + i, job, rho0=(0.5, 5.0))
        c["gnd"] = gnd
        cases.append(c)

    def fields(j, gnd):
        st = _state(evpg, j)
        if gnd:
            st[evpg.F_RHO_G1] = j.download(evpg.F_RHO_G1)
            st[evpg.F_RHO_G2] = j.download(evpg.F_RHO_G2)
        return st
    ref = []
    for c in cases:
        with evpg.Job(c["input"], c["rho0"], precision=precision, nr_mode=1, gnd=c["gnd"]) as j:
            ref.append(([j.increment(k) for k in range(4)], fields(j, c["gnd"])))
    jobs = [evpg.Job(c["input"], c["rho0"], precision=precision, nr_mode=1, gnd=c["gnd"]) for c in cases]
    try:
        its, _ = evpg.run_batched(jobs, [4, 4, 4], max_ticks=29)
        assert its == [r[0] for r in ref]
        for j, c, (_, st) in zip(jobs, cases, ref):
            got = fields(j, c["gnd"])
            for f, v in st.items():
                assert np.array_equal(got[f], v), f
        assert np.abs(ref[0][1][evpg.F_RHO_G1]).max() > 0
    finally:
        for j in jobs:
            j.close()


def test_radix16_stages(tmp_path):
    """Radix-16 Stockham stages (FP32) on the x axis, with other orders on y
    and z, separate passes, against the default radix orders: FP32-bulk
    results within the form's tolerance; radix 16 on the y axis is refused."""
    from conftest import rel_err
    from srx_gb300 import rve
    evpg = _evpg()
    grid = (32, 64, 64)
    job = rve.Job(n=grid, load="tension", rate=1e-3, strain_per_step=2e-4, n_steps=2)
    c = rve.make_case(str(tmp_path / "c"), grid, 6, 33, job, rho0=(0.5, 5.0))
    res = []
    for orders in (None, ([16, 2], [8, 8], [2, 4, 8])):
        with evpg.Job(c["input"], c["rho0"], precision=1, nr_mode=1) as j:
            j.set_fused(0)
            j.set_xpass(0)
            if orders:
                for ax, r in enumerate(orders):
                    j.set_radix(ax, r)
                assert [list(x) for x in j.schedule()["radix_xyz"]] == [list(o) for o in orders]
            its = [j.increment(k) for k in range(2)]
            res.append((its, j.download(evpg.F_SIG6), j.scalars()))
    with evpg.Job(c["input"], c["rho0"], precision=1, nr_mode=1) as j:
        with pytest.raises(evpg.EvpgError):
            j.set_radix(1, [4, 16])
    assert abs(sum(res[0][0]) - sum(res[1][0])) <= 2
    assert rel_err(res[1][2][7:16], res[0][2][7:16]) < 1e-5
    l2 = np.linalg.norm(res[1][1] - res[0][1]) / np.linalg.norm(res[0][1])
    assert l2 < 1e-4, l2


@pytest.mark.parametrize("n0", [32, 64, 128])
def test_warp_x_pass_equals_shared_memory_pass(tmp_path, n0):
    """The warp-register X pass (one warp per pencil, all six components in
    registers, inverse transforms from the bit-reversed order) against the
    shared-memory Stockham X pass on the same FP32-bulk increments: results
    within the form's tolerance, for 1, 2 and 4 elements per lane, with a
    mixed-radix y axis (18) and an odd z axis (15) beside the x axis."""
    from conftest import rel_err
    from srx_gb300 import rve
    evpg = _evpg()
    grid = (n0, 18, 15)
    job = rve.Job(n=grid, load="tension", rate=1e-3, strain_per_step=2e-4, n_steps=2)
    c = rve.make_case(str(tmp_path / "c"), grid, 6, 34, job, rho0=(0.5, 5.0))
    res = []
    for mode in (0, 1):
        with evpg.Job(c["input"], c["rho0"], precision=1, nr_mode=1) as j:
            j.set_xpass(mode)
            its = [j.increment(k) for k in range(2)]
            res.append((its, j.download(evpg.F_SIG6), j.scalars()))
    assert abs(sum(res[0][0]) - sum(res[1][0])) <= 2
    assert rel_err(res[1][2][7:16], res[0][2][7:16]) < 1e-5
    l2 = np.linalg.norm(res[1][1] - res[0][1]) / np.linalg.norm(res[0][1])
    assert l2 < 1e-4, l2


def test_deferred_antisymmetric_correction(tmp_path):
    """FP32 bulk with both warp-register passes (32^3) sums the antisymmetric
    part of the displacement-gradient correction (A12, A13, A23) in the
    spectrum during the equilibrium loop and transforms it once, at the end of
    the increment. Against the same shear increments with the shared-memory
    X pass, which transforms all nine components every iteration: the
    displacement gradient, the velocity gradient (whose antisymmetric part is
    the spin that reorients the lattice), the orientation and the stress
    within the form's tolerance."""
    from conftest import rel_err
    from srx_gb300 import rve
    evpg = _evpg()
    grid = (32, 32, 32)
    job = rve.Job(n=grid, load="shear", rate=1e-3, strain_per_step=1e-4, n_steps=2)
    c = rve.make_case(str(tmp_path / "c"), grid, 9, 77, job, rho0=(0.5, 5.0))
    res = []
    for mode in (1, 0):
        with evpg.Job(c["input"], c["rho0"], precision=1, nr_mode=1) as j:
            j.set_xpass(mode)
            assert j.variant()[0] > 0 and (j.variant()[1] > 0) == bool(mode)
            its = [j.increment(k) for k in range(2)]
            res.append((its, [j.download(f) for f in (evpg.F_DISGRAD, evpg.F_VELGRAD, evpg.F_TRANMAT,
                                                      evpg.F_SIG6)], j.scalars()))
    assert abs(sum(res[0][0]) - sum(res[1][0])) <= 2
    assert rel_err(res[0][2][7:16], res[1][2][7:16]) < 1e-5
    for a, b in zip(res[0][1], res[1][1]):
        l2 = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert l2 < 1e-4, l2
    # the antisymmetric part is not negligible here: somewhere in the RVE the
    # velocity gradient's spin reaches a percent of its symmetric part
    vg = res[0][1][1].reshape(-1, 3, 3)
    w = 0.5 * (vg - vg.transpose(0, 2, 1))
    assert np.abs(w).max() > 0.01 * np.abs(0.5 * (vg + vg.transpose(0, 2, 1))).max()
