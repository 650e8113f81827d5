"""CPU tests of the drop-in boundary: the C-ABI libraries load, export every
symbol the public header declares, the Python layer keeps the reference's
signatures, validates arguments before any native call, and fails loudly
(never falls back to a CPU path) when no GPU is present."""
import ctypes
import inspect
import os
import re

import numpy as np
import pytest

from conftest import PKG, ROOT, gpu_available

HEADER = os.path.join(ROOT, "include", "cilreg_gb300.h")


def _declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text)) - {"defined"})


def test_header_declares_the_reference_abi():
    syms = set(_declared_symbols())
    ref_gpu = {"TV_ROF_GPU_main", "TV_FGP_GPU_main", "TV_PD_GPU_main", "TV_SB_GPU_main", "TGV_GPU_main",
               "NonlDiff_GPU_main", "Diffus4th_GPU_main"}
    ref_cpu = {"TV_ROF_CPU_main", "TV_FGP_CPU_main", "PDTV_CPU_main", "SB_TV_CPU_main", "TGV_main",
               "Diffusion_CPU_main", "Diffus4th_CPU_main"}
    assert ref_gpu <= syms and ref_cpu <= syms


@pytest.mark.parametrize("lib", ["libcilregcuda.so", "libcilreg.so"])
def test_library_exports_every_declared_symbol(lib):
    path = os.path.join(PKG, "ccpi", "filters", lib)
    assert os.path.exists(path), f"{path} not built (run python build.py)"
    handle = ctypes.CDLL(path)
    missing = [s for s in _declared_symbols() if not hasattr(handle, s)]
    assert not missing, missing


def test_both_library_names_share_one_copy():
    """libcilreg.so forwards to libcilregcuda.so: an error recorded through one
    name is the one the other reports, and both count the same launches."""
    cpu = ctypes.CDLL(os.path.join(PKG, "ccpi", "filters", "libcilreg.so"))
    gpu = ctypes.CDLL(os.path.join(PKG, "ccpi", "filters", "libcilregcuda.so"))
    cpu.cilreg_prox_session_create.restype = ctypes.c_int
    assert cpu.cilreg_prox_session_create(None, 0, None, 0, 1, 1, 1, None) == -2
    gpu.cilreg_last_error.restype = ctypes.c_char_p
    assert b"null session pointer" in gpu.cilreg_last_error()
    cpu.cilreg_launch_count.restype = gpu.cilreg_launch_count.restype = ctypes.c_longlong
    assert cpu.cilreg_launch_count() == gpu.cilreg_launch_count()
    maps = open("/proc/self/maps").read()
    assert len({ln.split()[-1] for ln in maps.splitlines() if ln.endswith("libcilregcuda.so")}) == 1


def test_python_signatures_match_reference():
    from ccpi.filters import TV, diffusion, regularisersCuPy

    expect = {
        TV.TV_ROF_CPU: ["inputData", "regularisation_parameter", "iterationsNumb", "marching_step_parameter",
                        "tolerance_param", "out", "infovector"],
        TV.TV_FGP_CPU: ["inputData", "lambdaPar", "iterationsNumb", "epsil", "methodTV", "nonneg", "out",
                        "infovector"],
        TV.PDTV_CPU: ["inputData", "lambdaPar", "iterationsNumb", "epsil", "lipschitz_const", "methodTV", "nonneg",
                      "out", "infovector"],
        TV.SB_TV_CPU: ["inputData", "mu", "iter", "epsil", "methodTV", "out", "infovector"],
        TV.TGV_CPU: ["inputData", "lambdaPar", "alpha1", "alpha0", "iterationsNumb", "L2", "epsil", "out",
                     "infovector"],
        diffusion.NDF_CPU: ["inputData", "lambdaPar", "sigmaPar", "iterationsNumb", "tau", "penaltytype", "epsil",
                            "out", "infovector"],
        diffusion.Diffus4th_CPU: ["inputData", "lambdaPar", "sigmaPar", "iterationsNumb", "tau", "epsil", "out",
                                  "infovector"],
        TV.PDTV_GPU: ["Input", "lambdaPar", "iter", "epsil", "lipschitz_const", "methodTV", "nonneg", "gpu_device",
                      "Output", "infovector"],
        TV.SB_TV_GPU: ["inputData", "lambdaPar", "iterationsNumb", "epsil", "methodTV", "gpu_device", "out",
                       "infovector"],
        regularisersCuPy.ROF_TV: ["data", "regularisation_parameter", "iterations", "time_marching_parameter",
                                  "gpu_id"],
        regularisersCuPy.PD_TV: ["data", "regularisation_parameter", "iterations", "tolerance_param", "methodTV",
                                 "nonneg", "lipschitz_const", "gpu_id"],
    }
    for fn, names in expect.items():
        got = list(inspect.signature(fn).parameters)
        assert got[: len(names)] == names, (fn.__name__, got)


def test_device_dispatch_matches_reference():
    from ccpi.filters import regularisers as R

    with pytest.raises(KeyError):
        R.FGP_TV(np.zeros((4, 4), np.float32), 0.1, 1, 0.0, 0, 0, device="tpu")


@pytest.mark.parametrize(
    "bad, exc",
    [
        (np.zeros((8, 8), np.float64), TypeError),
        (np.zeros((8,), np.float32), ValueError),
        (np.zeros((2, 2, 2, 2), np.float32), ValueError),
        ([[0.0, 1.0]], TypeError),
    ],
)
def test_input_validation_precedes_native_calls(bad, exc):
    from ccpi.filters import regularisers as R

    with pytest.raises(exc):
        R.FGP_TV(bad, 0.1, 1, 0.0, 0, 0)


def test_output_validation():
    from ccpi.filters import regularisers as R

    x = np.zeros((8, 8), np.float32)
    with pytest.raises(ValueError):
        R.ROF_TV(x, 0.1, 1, 0.001, 0.0, out=np.zeros((8, 9), np.float32))
    with pytest.raises(TypeError):
        R.ROF_TV(x, 0.1, 1, 0.001, 0.0, infovector=np.zeros(1, np.float32))


def test_out_of_scope_regularisers_raise():
    from ccpi.filters import regularisers as R

    for fn in (R.PatchSelect, R.NLTV, R.TNV):
        with pytest.raises(NotImplementedError):
            fn(np.zeros((4, 4), np.float32))


@pytest.mark.skipif(gpu_available(), reason="checks behaviour without a GPU")
def test_no_gpu_fails_loudly():
    from ccpi.filters import regularisers as R
    from ccpi.filters.utils import RegulariserError

    x = np.ones((8, 8), np.float32)
    for dev in ("cpu", "gpu"):
        with pytest.raises(RegulariserError) as e:
            R.FGP_TV(x, 0.1, 5, 0.0, 0, 0, device=dev)
        assert e.value.status == -3


def test_invalid_dims_rejected_by_the_library():
    from ccpi.filters.utils import cilregcuda

    f = (ctypes.c_float * 4)()
    st = cilregcuda.TV_FGP_GPU_main(f, f, f, 0.1, 1, 0.0, 0, 0, 0, 0, 2, 1)
    assert st == -2
    assert b"invalid dimensions" in cilregcuda.cilreg_last_error()


def test_product_never_imports_the_oracle():
    """The product path must not route through the CPU checker."""
    for dirpath, _, files in os.walk(PKG):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text and "liboracle" not in text and "cilreg_port" not in text, f
