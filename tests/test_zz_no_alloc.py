"""The allocation-free Green-operator correction against the context path.

evpg_green_correction_noalloc serves callers that cannot allocate device
memory while they run (their device memory belongs to another allocator, or
their footprint is fixed at load time); its scratch is a static device array.
This checks it, through the C ABI and on two calls in a row, against the
correction the context path applies in the first two equilibrium iterations
of an increment (DisGrad after minus before, minus the macro term), at the
field tolerance of the other GPU tests (1e-8 of the field's largest entry).
The file is collected last so a failure here leaves every other test run."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden, rel_err, write_spec_case

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-8
R2, R3, R6 = 0.70710678118654744, 0.57735026918962584, 0.40824829046386304


def _to_b6(t):
    """[N][3][3] -> [6][N] in the B basis (kinematics.c:62-69)."""
    t = t.reshape(-1, 3, 3)
    return np.stack([R2 * (t[:, 1, 1] - t[:, 0, 0]),
                     R6 * (2 * t[:, 2, 2] - t[:, 0, 0] - t[:, 1, 1]),
                     R2 * (t[:, 1, 2] + t[:, 2, 1]), R2 * (t[:, 0, 2] + t[:, 2, 0]),
                     R2 * (t[:, 0, 1] + t[:, 1, 0]), R3 * (t[:, 0, 0] + t[:, 1, 1] + t[:, 2, 2])])


def _from_9(q):
    """[9][N] (B basis + A12, A13, A23) -> [N][3][3]."""
    v = q
    t = np.zeros((q.shape[1], 3, 3))
    t[:, 0, 0] = -R2 * v[0] - R6 * v[1] + R3 * v[5]
    t[:, 1, 1] = R2 * v[0] - R6 * v[1] + R3 * v[5]
    t[:, 2, 2] = 2 * R6 * v[1] + R3 * v[5]
    t[:, 1, 2] = t[:, 2, 1] = R2 * v[2]
    t[:, 0, 2] = t[:, 2, 0] = R2 * v[3]
    t[:, 0, 1] = t[:, 1, 0] = R2 * v[4]
    t[:, 0, 1] += v[6]; t[:, 1, 0] -= v[6]
    t[:, 0, 2] += v[7]; t[:, 2, 0] -= v[7]
    t[:, 1, 2] += v[8]; t[:, 2, 1] -= v[8]
    return t


def _case(tmp_path, grid, elast_bc):
    """The 16^3 golden RVE, or a seeded Voronoi RVE on another grid: 32^3 is
    the largest half spectrum the scratch holds, 64x16x8 puts an axis at the
    length limit (where the x pass takes its largest shared-memory tile),
    12x10x9 has radix-3/5 stages and odd lengths. elast_bc 0 sets the k = 0
    term to -S0:sigma_hat(0) instead of zero."""
    if grid == "golden16":
        z, spec = golden("voronoi16_ls")
        return write_spec_case(spec, tmp_path / "case"), list(spec["n"])
    from srx_gb300 import rve
    job = rve.Job(n=grid, n_steps=1, elast_bc=elast_bc)
    return rve.make_case(str(tmp_path / "case"), grid, 6, 31, job), list(grid)


@pytest.mark.parametrize("grid,elast_bc", [("golden16", 1), ((32, 32, 32), 1), ((64, 16, 8), 0),
                                           ((12, 10, 9), 0), ((12, 10, 9), 1)])
def test_noalloc_green_correction_matches_context_path(tmp_path, grid, elast_bc):
    import torch
    from srx_gb300 import build, evpg
    build.build()
    L = evpg.lib()
    L.evpg_green_correction_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                                C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32,
                                                C.c_void_p]
    case, n = _case(tmp_path, grid, elast_bc)
    N = int(np.prod(n))
    with evpg.Job(case["input"], nr_mode=1) as j:
        # reference-stiffness tensors of this RVE, from the oracle's set-up
        from conftest import Oracle
        o = Oracle()
        h = o.open(case["input"])
        c066 = o.field(h, "C066", 36).reshape(6, 6).copy()
        s0 = o.field(h, "S0", 81).copy()
        o.L.evo_close(h)
        # C0 from C066 (chg_basis opt 3, kinematics.c:70-77)
        B = np.zeros((6, 3, 3))
        B[0, 0, 0], B[0, 1, 1] = -R2, R2
        B[1, 0, 0] = B[1, 1, 1] = -R6; B[1, 2, 2] = 2 * R6
        B[2, 1, 2] = B[2, 2, 1] = R2
        B[3, 0, 2] = B[3, 2, 0] = R2
        B[4, 0, 1] = B[4, 1, 0] = R2
        B[5, 0, 0] = B[5, 1, 1] = B[5, 2, 2] = R3
        c0 = np.einsum("ij,iab,jcd->abcd", c066, B, B).reshape(-1).copy()
        ctx = j.ctx
        udt = (C.c_double * 9)(*[0, 0, 0, 0, 0, 0, 0, 0, 2e-4])
        zero = (C.c_double * 9)()
        evpg.check(L.evpg_increment_begin(ctx, udt, 0, zero, 0.0))
        sig_before = j.download(evpg.F_SIG)
        dg0 = j.download(evpg.F_DISGRAD)
        out = evpg.IterOut()
        evpg.check(L.evpg_equilibrium_iteration(ctx, 1e-4, C.byref(out)))
        dg1 = j.download(evpg.F_DISGRAD)
        sig1 = j.download(evpg.F_SIG)
        dE1 = np.array(out.ddisgrad[:]).reshape(3, 3)
        evpg.check(L.evpg_equilibrium_iteration(ctx, 1e-4, C.byref(out)))
        dg2 = j.download(evpg.F_DISGRAD)
    ref1 = (dg1 - dg0).reshape(N, 3, 3)
    ref2 = (dg2 - dg1).reshape(N, 3, 3) - dE1[None]

    dev = torch.device("cuda:0")
    du = torch.empty(9 * N, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    c0p = (C.c_double * 81)(*c0)
    s0p = (C.c_double * 81)(*s0)
    for sig, ref in ((sig_before, ref1), (sig1, ref2)):
        s6 = torch.from_numpy(np.ascontiguousarray(_to_b6(sig)).reshape(-1)).to(dev)
        st = L.evpg_green_correction_noalloc(s6.data_ptr(), du.data_ptr(), n[0], n[1], n[2], c0p, s0p,
                                             elast_bc, C.c_void_p(stream.cuda_stream))
        assert st == 0, st
        torch.cuda.synchronize()
        got = _from_9(du.cpu().numpy().reshape(9, N))
        assert rel_err(got, ref) < FIELD_TOL


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    from srx_gb300 import build, evpg
    build.build()
    L = evpg.lib()
    L.evpg_green_correction_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                                C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32,
                                                C.c_void_p]
    x = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    c = (C.c_double * 81)()
    assert L.evpg_green_correction_noalloc(x.data_ptr(), x.data_ptr(), 64, 64, 64, c, c, 1, None) == 1
    assert L.evpg_green_correction_noalloc(x.data_ptr(), x.data_ptr(), 128, 2, 2, c, c, 1, None) == 1
