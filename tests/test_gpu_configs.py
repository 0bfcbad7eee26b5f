"""Multi-increment parity on the benchmark configurations, against runs of the
reference itself (golden fixtures written by tests/golden/make_golden.py from
the reference's own sources):

* cfg0_32_run  the 32^3 / 27-grain configuration over its whole load path
               (50 increments of 2e-4 strain);
* cfg1_64_ls   the 64^3 / 125-grain configuration, first 5 increments;
* cfg2_128_ls  the 128^3 / 1000-grain precision-form configuration with
               per-grain log-uniform initial density (the benchmark's own
               RVE), first 2 increments.

FP64 plain form: identical equilibrium iteration counts in every increment;
vm.out and dd.out rows of every increment column by column at print
precision (2e-6 of the column's largest entry); stress, SSD density and
accumulated slip at the stored increments within 1e-8 of each field's
largest entry.

FP32-bulk form: the fused plane kernels and the warp-register X pass at the
grid's lane layout (32-, 64- and 128-point); identical iteration counts;
macroscopic von Mises stress within 1e-4 relative in every increment; stress
and SSD density fields within 1e-3 (L2) at the stored increments."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, col_err, golden, rel_err, write_spec_case

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-8
PRINT_TOL = 2e-6
CASES = [pytest.param(n, marks=pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, n + ".npz")),
                                                 reason="golden fixture %s.npz not generated" % n))
         for n in ("cfg0_32_run", "cfg1_64_ls", "cfg2_128_ls")]
VARIANT = {32: (1, 1), 64: (2, 2), 128: (4, 4)}


def _evpg():
    from srx_gb300 import build, evpg
    build.build()
    return evpg


def _run(evpg, z, spec, case, precision):
    """Increments of the spec through the job API; per increment the vm.out
    and dd.out rows (from the job's scalars), and at the stored increments
    the stress (.iout order 11,22,33,23,13,12), SSD density and accumulated
    slip of the stored voxels."""
    idx = z["idx"]
    keep = set(int(s) for s in z["keep"])
    its, vm, dd, fields = [], [], [], {}
    with evpg.Job(case["input"], case.get("rho0"), precision=precision, nr_mode=evpg.NR_LINESEARCH) as j:
        variant = j.variant()
        for k in range(spec["steps"]):
            its.append(j.increment(k))
            s = j.scalars()
            vm.append(s[0:7])
            r = s[25:33]
            dd.append([s[0], s[1], r[2], r[3], r[5], r[7], r[6]])
            if k in keep:
                fields["sig_%d" % k] = j.download(evpg.F_SIG6)[idx]
                fields["rho_s_%d" % k] = j.download(evpg.F_RHO_S)[idx]
                fields["gam_acum_%d" % k] = j.download(evpg.F_GAM_ACUM)[idx]
    return its, np.array(vm), np.array(dd), fields, variant


def _l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", CASES)
def test_fp64_matches_reference_every_increment(tmp_path, name):
    evpg = _evpg()
    z, spec = golden(name)
    case = write_spec_case(spec, tmp_path / "case")
    its, vm, dd, f, _ = _run(evpg, z, spec, case, evpg.FP64)
    assert its == list(z["iters"])
    assert col_err(vm, z["vm"]) < PRINT_TOL
    assert col_err(dd, z["dd"]) < PRINT_TOL
    for s in z["keep"]:
        for k in ("sig", "rho_s", "gam_acum"):
            assert rel_err(f["%s_%d" % (k, s)], z["%s_%d" % (k, s)]) < FIELD_TOL, (k, int(s))


@pytest.mark.parametrize("name", CASES)
def test_fp32_bulk_headline_kernels_within_stated_error(tmp_path, name):
    evpg = _evpg()
    z, spec = golden(name)
    case = write_spec_case(spec, tmp_path / "case")
    its, vm, dd, f, variant = _run(evpg, z, spec, case, evpg.FP32_BULK)
    assert variant == VARIANT[spec["n"][0]]
    assert its == list(z["iters"])
    svm_err = np.abs(vm[:, 5] - z["vm"][:, 5]) / np.abs(z["vm"][:, 5])
    assert svm_err.max() < 1e-4, svm_err.max()
    for s in z["keep"]:
        for k in ("sig", "rho_s"):
            e = _l2(f["%s_%d" % (k, s)], z["%s_%d" % (k, s)])
            assert e < 1e-3, (k, int(s), e)
