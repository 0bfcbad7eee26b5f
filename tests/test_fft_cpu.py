"""The oracle's CPU DFT (stand-in for FFTW 2 at evolution.c:1163,1195)
against numpy.fft."""
import ctypes as C

import numpy as np
import pytest

from conftest import ORACLE_LIB, build_oracle

SHAPES = [(8, 8, 8), (16, 12, 10), (7, 9, 11), (48, 32, 5), (3, 5, 25), (128, 4, 6),
          (96, 2, 3), (1, 1, 64), (2, 2, 2), (13, 1, 1), (49, 1, 1)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("sign", [-1, 1])
def test_fft3d_matches_numpy(shape, sign):
    build_oracle()
    L = C.CDLL(ORACLE_LIB)
    L.srx_fft3d.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
    rng = np.random.default_rng(abs(hash(shape)) % 1000 + (sign > 0))
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    a = np.ascontiguousarray(x.copy())
    assert L.srx_fft3d(a.ctypes.data, *shape, sign) == 0
    ref = np.fft.fftn(x) if sign < 0 else np.fft.ifftn(x) * np.prod(shape)
    assert np.max(np.abs(a - ref)) <= 2e-15 * max(1.0, np.log2(np.prod(shape))) * np.max(np.abs(ref))
