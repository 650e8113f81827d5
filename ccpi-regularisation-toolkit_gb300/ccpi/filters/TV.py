"""Total-variation family: same functions and signatures as the reference's
src/Python/ccpi/filters/TV.py (ROF, FGP, PD, SB, TGV, LLT-ROF, FGP-dTV and the
TV energy diagnostic).

``*_CPU`` functions call the ``*_CPU_main`` entry points of ``libcilreg.so``,
which in this build execute on the GPU named by ``CILREG_GPU_DEVICE``
(default 0); ``*_GPU`` functions call ``*_GPU_main`` with an explicit device.
Every call raises on a failure status instead of returning garbage.
"""
import ctypes

import numpy as np

from ._marshal import as_info, as_input, as_output, dims, ptr
from .utils import check_status, cilreg, cilregcuda


# ---------------------------------------------------------------------------
# C-OMP argument lists (TV.py:8-250 of the reference)
def TV_ROF_CPU(inputData, regularisation_parameter, iterationsNumb, marching_step_parameter, tolerance_param,
               out=None, infovector=None):
    """ROF-TV explicit gradient flow (ROF_TV_core.c:50).  ``regularisation_parameter``
    may be a scalar or a float32 array of the input's shape (per-voxel lambda)."""
    a = as_input(inputData)
    out = as_output(out, a)
    info = as_info(infovector)
    if np.ndim(regularisation_parameter) == 0:
        lam = np.array([regularisation_parameter], dtype=np.float32)
        is_arr = 0
    else:
        lam = np.ascontiguousarray(regularisation_parameter, dtype=np.float32)
        if lam.shape != a.shape:
            raise ValueError("per-voxel regularisation_parameter must match the input shape")
        is_arr = 1
    st = cilreg.TV_ROF_CPU_main(ptr(a), ptr(out), ptr(info), ptr(lam), is_arr, int(iterationsNumb),
                                float(marching_step_parameter), float(tolerance_param), *dims(a))
    check_status(st, cilreg)
    return out


def TV_FGP_CPU(inputData, lambdaPar, iterationsNumb, epsil, methodTV, nonneg, out=None, infovector=None):
    """FGP-TV (FGP_TV_core.c:40)."""
    a = as_input(inputData)
    out = as_output(out, a)
    info = as_info(infovector)
    st = cilreg.TV_FGP_CPU_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), int(iterationsNumb), float(epsil),
                                int(methodTV), int(nonneg), *dims(a))
    check_status(st, cilreg)
    return out


def PDTV_CPU(inputData, lambdaPar, iterationsNumb, epsil, lipschitz_const, methodTV, nonneg, out=None,
             infovector=None):
    """Primal-dual TV (PD_TV_core.c:40)."""
    a = as_input(inputData)
    out = as_output(out, a)
    info = as_info(infovector)
    st = cilreg.PDTV_CPU_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), int(iterationsNumb), float(epsil),
                              float(lipschitz_const), int(methodTV), int(nonneg), *dims(a))
    check_status(st, cilreg)
    return out


def SB_TV_CPU(inputData, mu, iter, epsil, methodTV, out=None, infovector=None):
    """Split-Bregman TV (SB_TV_core.c:38)."""
    a = as_input(inputData)
    out = as_output(out, a)
    info = as_info(infovector)
    st = cilreg.SB_TV_CPU_main(ptr(a), ptr(out), ptr(info), float(mu), int(iter), float(epsil), int(methodTV),
                               *dims(a))
    check_status(st, cilreg)
    return out


def TGV_CPU(inputData, lambdaPar, alpha1, alpha0, iterationsNumb, L2, epsil, out=None, infovector=None):
    """TGV^2 primal-dual (TGV_core.c:43)."""
    a = as_input(inputData)
    out = as_output(out, a)
    info = as_info(infovector)
    st = cilreg.TGV_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), float(alpha1), float(alpha0),
                         int(iterationsNumb), float(L2), float(epsil), *dims(a))
    check_status(st, cilreg)
    return out


# ---------------------------------------------------------------------------
# GPU argument lists (TV.py:470-733 of the reference)
def _dev(gpu_device):
    return 0 if gpu_device == "gpu" else int(gpu_device)


def TV_ROF_GPU(inputData, regularisation_parameter, iterationsNumb, marching_step_parameter, tolerance_param,
               gpu_device, out=None, infovector=None):
    a = as_input(inputData)
    out = as_output(out, a, zero_init=int(iterationsNumb) <= 0)
    info = as_info(infovector)
    st = cilregcuda.TV_ROF_GPU_main(ptr(a), ptr(out), ptr(info), float(regularisation_parameter),
                                    int(iterationsNumb), float(marching_step_parameter), float(tolerance_param),
                                    _dev(gpu_device), *dims(a))
    check_status(st)
    return out


def TV_FGP_GPU(inputData, lambdaPar, iterationsNumb, epsil, methodTV, nonneg, gpu_device, out=None,
               infovector=None):
    a = as_input(inputData)
    out = as_output(out, a, zero_init=int(iterationsNumb) <= 0)
    info = as_info(infovector)
    st = cilregcuda.TV_FGP_GPU_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), int(iterationsNumb),
                                    float(epsil), int(methodTV), int(nonneg), _dev(gpu_device), *dims(a))
    check_status(st)
    return out


def PDTV_GPU(Input, lambdaPar, iter, epsil, lipschitz_const, methodTV, nonneg, gpu_device, Output=None,
             infovector=None):
    a = as_input(Input)
    out = as_output(Output, a, zero_init=int(iter) <= 0)
    info = as_info(infovector)
    st = cilregcuda.TV_PD_GPU_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), int(iter), float(epsil),
                                   float(lipschitz_const), int(methodTV), int(nonneg), _dev(gpu_device), *dims(a))
    check_status(st)
    return out


def SB_TV_GPU(inputData, lambdaPar, iterationsNumb, epsil, methodTV, gpu_device, out=None, infovector=None):
    a = as_input(inputData)
    out = as_output(out, a, zero_init=int(iterationsNumb) <= 0)
    info = as_info(infovector)
    st = cilregcuda.TV_SB_GPU_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), int(iterationsNumb),
                                   float(epsil), int(methodTV), _dev(gpu_device), *dims(a))
    check_status(st)
    return out


def TGV_GPU(inputData, lambdaPar, alpha1, alpha0, iterationsNumb, L2, epsil, gpu_device, out=None,
            infovector=None):
    """TGV on the GPU.  Unlike the reference (TV.py:722-725), the dims are
    passed with dimX fastest, so GPU and CPU results agree for every shape."""
    a = as_input(inputData)
    out = as_output(out, a, zero_init=int(iterationsNumb) <= 0)
    info = as_info(infovector)
    st = cilregcuda.TGV_GPU_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), float(alpha1), float(alpha0),
                                 int(iterationsNumb), float(L2), float(epsil), _dev(gpu_device), *dims(a))
    check_status(st)
    return out


# ---------------------------------------------------------------------------
# Regularisers of the reference that this build does not provide.  They are
# importable so that code importing them keeps loading, and raise on use.
def _not_provided(name):
    def f(*args, **kwargs):
        raise NotImplementedError(f"{name} is not part of the GB300 regulariser build")

    f.__name__ = name
    return f


PatchSelect_CPU = _not_provided("PatchSelect")
PatchSelect_GPU = _not_provided("PatchSelect")
NLTV = _not_provided("NLTV")
TNV = _not_provided("TNV")


# ---------------------------------------------------------------------------
# LLT-ROF, FGP-dTV and the TV energy (TV.py:174-250, 252-290, 421-459,
# 650-689, 735-780 of the reference)
def _as_like(b, a, name):
    b = as_input(b)
    if b.shape != a.shape:
        raise ValueError(f"{name} has shape {b.shape}, expected {a.shape}")
    return b


def LLT_ROF_CPU(inputData, lambdaROF, lambdaLLT, iterationsNumb, tau, epsil, out=None, infovector=None):
    """LLT-ROF (LLT_ROF_core.c:54): fourth-order LLT plus ROF-TV explicit flow."""
    a = as_input(inputData)
    out = as_output(out, a)
    info = as_info(infovector)
    st = cilreg.LLT_ROF_CPU_main(ptr(a), ptr(out), ptr(info), float(lambdaROF), float(lambdaLLT),
                                 int(iterationsNumb), float(tau), float(epsil), *dims(a))
    check_status(st, cilreg)
    return out


def LLT_ROF_GPU(inputData, lambdaROF, lambdaLLT, iterationsNumb, tau, epsil, gpu_device, out=None,
                infovector=None):
    a = as_input(inputData)
    out = as_output(out, a, zero_init=int(iterationsNumb) <= 0)
    info = as_info(infovector)
    st = cilregcuda.LLT_ROF_GPU_main(ptr(a), ptr(out), ptr(info), float(lambdaROF), float(lambdaLLT),
                                     int(iterationsNumb), float(tau), float(epsil), _dev(gpu_device), *dims(a))
    check_status(st)
    return out


def dTV_FGP_CPU(inputData, inputRef, lambdaPar, iterationsNumb, epsil, eta, methodTV, nonneg, out=None,
                infovector=None):
    """FGP-dTV (FGP_dTV_core.c:46): FGP on the directional TV guided by inputRef."""
    a = as_input(inputData)
    r = _as_like(inputRef, a, "inputRef")
    out = as_output(out, a)
    info = as_info(infovector)
    st = cilreg.dTV_FGP_CPU_main(ptr(a), ptr(r), ptr(out), ptr(info), float(lambdaPar), int(iterationsNumb),
                                 float(epsil), float(eta), int(methodTV), int(nonneg), *dims(a))
    check_status(st, cilreg)
    return out


def dTV_FGP_GPU(inputData, inputRef, lambdaPar, iterationsNumb, epsil, eta, methodTV, nonneg, gpu_device,
                out=None, infovector=None):
    a = as_input(inputData)
    r = _as_like(inputRef, a, "inputRef")
    out = as_output(out, a, zero_init=int(iterationsNumb) <= 0)
    info = as_info(infovector)
    st = cilregcuda.dTV_FGP_GPU_main(ptr(a), ptr(r), ptr(out), ptr(info), float(lambdaPar), int(iterationsNumb),
                                     float(epsil), float(eta), int(methodTV), int(nonneg), _dev(gpu_device),
                                     *dims(a))
    check_status(st)
    return out


def TV_ENERGY(U, U0, lambdaPar, type, E_val=None):
    """TV energy (utils.c:60-117): type 1 gives 2 lambda TV(U) + |U - U0|^2,
    type 2 gives 2 lambda TV(U).  Returns a float32 array of one element."""
    u = as_input(U)
    u0 = _as_like(U0, u, "U0")
    if E_val is None:
        E_val = np.zeros((1,), dtype=np.float32)
    elif not isinstance(E_val, np.ndarray) or E_val.dtype != np.float32 or E_val.size < 1:
        raise TypeError("E_val must be a float32 ndarray with at least one element")
    if int(type) not in (1, 2):
        raise ValueError(f"TV_ENERGY: type must be 1 or 2, got {type}")
    if u.ndim == 2:
        r = cilreg.TV_energy2D(ptr(u), ptr(u0), ptr(E_val), float(lambdaPar), int(type), u.shape[1], u.shape[0])
    else:
        r = cilreg.TV_energy3D(ptr(u), ptr(u0), ptr(E_val), float(lambdaPar), int(type), u.shape[2], u.shape[1],
                               u.shape[0])
    if np.isnan(r):
        check_status(-1, cilreg)
    return E_val
