"""The kernels' own reciprocal against CUDA's correctly rounded one.

The two-voxel fourth-order diffusion kernel forms its two reciprocals as the
hardware's approximate reciprocal refined by one Newton-Raphson step
(pair.cuh, rcp2).  cilreg_selftest_reciprocal evaluates it on the device next
to CUDA's IEEE reciprocal (__frcp_rn); over every mantissa of one binade and
random normal values of both signs whose reciprocals are normal, the two
differ by at most one unit in the last place.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import PKG

pytestmark = pytest.mark.gpu


def _probe(x):
    lib = ctypes.CDLL(os.path.join(PKG, "ccpi", "filters", "libcilregcuda.so"))
    fp = ctypes.POINTER(ctypes.c_float)
    lib.cilreg_selftest_reciprocal.argtypes = [ctypes.c_int, fp, fp, fp, ctypes.c_longlong]
    lib.cilreg_selftest_reciprocal.restype = ctypes.c_int
    lib.cilreg_last_error.restype = ctypes.c_char_p
    x = np.ascontiguousarray(x, np.float32)
    approx, ieee = np.empty_like(x), np.empty_like(x)
    st = lib.cilreg_selftest_reciprocal(0, x.ctypes.data_as(fp), approx.ctypes.data_as(fp),
                                        ieee.ctypes.data_as(fp), x.size)
    assert st == 0, lib.cilreg_last_error()
    return approx, ieee


def test_newton_reciprocal_within_one_ulp_of_ieee():
    binade = (np.arange(1 << 23, dtype=np.uint32) | np.uint32(127 << 23)).view(np.float32)  # [1, 2)
    rng = np.random.default_rng(12)
    e = rng.integers(-125, 126, 4_000_000)
    m = rng.random(e.size) + 1.0
    wide = (np.ldexp(m, e) * np.where(rng.random(e.size) < 0.5, -1.0, 1.0)).astype(np.float32)
    wide = wide[(np.abs(wide) >= np.float32(2.0 ** -125)) & (np.abs(wide) <= np.float32(2.0 ** 125))]
    x = np.concatenate([binade, wide, np.float32([1e-7, 1.0, 3.0, 7.0, 1e7])])
    approx, ieee = _probe(x)
    # CUDA's reciprocal is the correctly rounded one
    np.testing.assert_array_equal(ieee, (1.0 / x.astype(np.float64)).astype(np.float32))
    ulps = np.abs(approx.view(np.int32).astype(np.int64) - ieee.view(np.int32).astype(np.int64))
    assert ulps.max() <= 1
    # and it is the rounded value almost always
    assert np.mean(ulps == 0) > 0.99
