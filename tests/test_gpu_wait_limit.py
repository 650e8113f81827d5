"""The bounded waits of the tensor-copy kernels run out and report it.

The kernels that stage their inputs by tensor copies wait on a stage's
mbarrier a bounded number of times, then record a failure that the host
turns into a failed call.  cilreg_selftest_wait_limit makes such a wait run
out on purpose (an mbarrier armed for bytes that no copy delivers, no copy in
flight) and checks that the device still runs work afterwards; the regular
calls that follow must still succeed.
"""
import ctypes
import os
import time

import numpy as np
import pytest

from conftest import PKG

pytestmark = pytest.mark.gpu


def test_wait_runs_out_and_the_device_stays_usable():
    from ccpi.filters.regularisers import FGP_TV

    lib = ctypes.CDLL(os.path.join(PKG, "ccpi", "filters", "libcilregcuda.so"))
    lib.cilreg_selftest_wait_limit.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.cilreg_selftest_wait_limit.restype = ctypes.c_int
    lib.cilreg_last_error.restype = ctypes.c_char_p
    ran_out = ctypes.c_int(-1)
    t0 = time.perf_counter()
    st = lib.cilreg_selftest_wait_limit(0, ctypes.byref(ran_out))
    dt = time.perf_counter() - t0
    assert st == 0, lib.cilreg_last_error()
    assert ran_out.value == 1
    assert dt < 60.0  # about a second of tries
    x = np.random.default_rng(3).random((12, 20, 24)).astype(np.float32)
    out = FGP_TV(x, 0.05, 10, 0.0, 0, 1, device="gpu")
    assert np.isfinite(out).all()


def test_persistent_batch_wait_runs_out_and_the_device_stays_usable():
    """The persistent batched kernel's dependency waits: a launch whose work
    items all wait for an iteration that is never released gives up after
    its poll limit, reports it, and the device keeps working."""
    from ccpi.filters.batch import FGP_TV_batch

    lib = ctypes.CDLL(os.path.join(PKG, "ccpi", "filters", "libcilregcuda.so"))
    lib.cilreg_selftest_batch_wait.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.cilreg_selftest_batch_wait.restype = ctypes.c_int
    lib.cilreg_last_error.restype = ctypes.c_char_p
    ran_out = ctypes.c_int(-1)
    t0 = time.perf_counter()
    st = lib.cilreg_selftest_batch_wait(0, ctypes.byref(ran_out))
    assert st == 0, lib.cilreg_last_error()
    assert ran_out.value == 1
    assert time.perf_counter() - t0 < 60.0
    vols = [np.random.default_rng(4).random((10, 12, 14)).astype(np.float32) for _ in range(3)]
    outs = FGP_TV_batch(vols, 0.05, 12)
    assert all(np.isfinite(o).all() for o in outs)
