"""The allocation-free ROF entry point, cilreg_rof_tv_dev_noalloc.

It exists for callers that cannot allocate device memory when they
regularise (a framework whose own allocator already holds the GPU's memory,
or a real-time path that forbids allocation after start-up); it keeps its
scratch in one fixed array inside the library.  This test calls it through
the C ABI and checks it against the allocating entry point, cilreg_rof_tv_dev,
twice in a row (the second call must not see state left by the first).

The file is named so that pytest collects it last: the library's fixed
68 MiB device array is then mapped only after every other GPU test has run,
and a failure here cannot stop a run with -x before the rest of the suite.
Its tests pass alone in a fresh process as well as after the others (they
depend on no other test's state).
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import PKG, rel_tol

pytestmark = pytest.mark.gpu

_P = ctypes.POINTER(ctypes.c_float)
_ARGS = [ctypes.c_void_p, ctypes.c_void_p, _P, ctypes.c_void_p, ctypes.c_float, ctypes.c_int, ctypes.c_float,
         ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]


def _lib():
    lib = ctypes.CDLL(os.path.join(PKG, "ccpi", "filters", "libcilregcuda.so"))
    for name in ("cilreg_rof_tv_dev", "cilreg_rof_tv_dev_noalloc"):
        getattr(lib, name).argtypes = _ARGS
        getattr(lib, name).restype = ctypes.c_int
    lib.cilreg_last_error.restype = ctypes.c_char_p
    return lib


def _run(lib, name, x, lam, iters, tau, epsil, stream, lam_map=None):
    import torch

    d_in = torch.from_numpy(x).cuda()
    d_out = torch.empty_like(d_in)
    d_lam = torch.from_numpy(lam_map).cuda() if lam_map is not None else None
    info = np.zeros(2, np.float32)
    dims = list(x.shape)[::-1] + ([1] if x.ndim == 2 else [])
    st = getattr(lib, name)(d_in.data_ptr(), d_out.data_ptr(), info.ctypes.data_as(_P),
                            d_lam.data_ptr() if d_lam is not None else None, lam, iters, tau, epsil, *dims, stream)
    assert st == 0, lib.cilreg_last_error()
    torch.cuda.synchronize()
    return d_out.cpu().numpy(), info


@pytest.mark.parametrize(
    "shape, iters, epsil, lam_map",
    [((40, 24, 30), 60, 0.0, False), ((48, 64), 300, 1e-3, False), ((20, 33, 17), 200, 5e-4, False),
     ((64, 80), 120, 0.0, False), ((18, 26, 34), 90, 1e-3, True)],
    ids=["3d_fixed", "2d_stop", "3d_stop", "2d_fixed", "3d_lambda_map"],
)
def test_noalloc_matches_allocating_entry_point(shape, iters, epsil, lam_map):
    import torch

    lib = _lib()
    rng = np.random.default_rng(3)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # two calls in a row through the shared scratch
        x = (rng.random(shape) + (call * 0.25)).astype(np.float32)
        lm = (0.01 + 0.03 * rng.random(shape)).astype(np.float32) if lam_map else None
        ref, ref_info = _run(lib, "cilreg_rof_tv_dev", x, 0.02, iters, 0.001, epsil, stream, lm)
        got, info = _run(lib, "cilreg_rof_tv_dev_noalloc", x, 0.02, iters, 0.001, epsil, stream, lm)
        assert np.max(np.abs(got - ref)) <= rel_tol(ref, 1e-4), f"call {call}"
        assert int(info[0]) == int(ref_info[0]), f"call {call}"
        assert abs(float(info[1]) - float(ref_info[1])) <= 1e-6 + 1e-3 * abs(float(ref_info[1]))


def test_noalloc_rejects_oversize_input():
    import torch

    lib = _lib()
    d = torch.zeros(16, device="cuda")
    e = torch.zeros(16, device="cuda")
    info = np.zeros(2, np.float32)
    # 257^3 voxels exceed the 2^24-voxel limit; the call is refused before any GPU work
    st = lib.cilreg_rof_tv_dev_noalloc(d.data_ptr(), e.data_ptr(), info.ctypes.data_as(_P), None, 0.02, 5, 0.001,
                                       0.0, 257, 257, 257, torch.cuda.current_stream().cuda_stream)
    assert st == -2
    assert b"no-allocation limit" in lib.cilreg_last_error()
