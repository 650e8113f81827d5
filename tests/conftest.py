import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ccpi-regularisation-toolkit_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _autotune_cache_in_tmp(tmp_path_factory):
    """The batch autotuner's file cache goes to a temporary directory, not the
    user's home, while the tests run."""
    if "CILREG_AUTOTUNE_CACHE" not in os.environ:
        os.environ["CILREG_AUTOTUNE_CACHE"] = str(tmp_path_factory.mktemp("tune") / "autotune.tsv")
    yield


@pytest.fixture(scope="session", autouse=True)
def _built_oracle():
    """The oracle port is test infrastructure: (re)build it once per session."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    yield


@pytest.fixture(scope="session")
def golden():
    path = os.path.join(ROOT, "tests", "golden", "reference_outputs.npz")
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def rel_tol(ref: np.ndarray, frac: float = 1e-4) -> float:
    """Tolerance ``frac`` of the data range (the parity bar: max-abs <= 1e-4 * range)."""
    rng = float(np.max(ref) - np.min(ref))
    return frac * max(rng, 1e-12)
