"""Device-array regularisers: the reference's src/Python/ccpi/filters/regularisersCuPy.py
(ROF_TV :35-40, PD_TV :130-138) with the same signatures, extended to all
seven regularisers, LLT-ROF, FGP-dTV and the TV energy.

Inputs are device arrays already resident on the GPU: CuPy arrays, torch
CUDA tensors, or any object exposing ``__cuda_array_interface__`` (float32,
C-contiguous, 2D or 3D).  Results are returned as a new array of the same
kind (torch tensor for a torch input, CuPy array for a CuPy input).  Work
runs on the caller's current stream of that library; no host copies happen.
Each function also accepts ``infovector=`` (a 2-element float32 numpy array)
to receive [iterations run, last relative change].
"""
from __future__ import annotations

import numpy as np

from .utils import check_status, cilregcuda

__all__ = ["ROF_TV", "PD_TV", "FGP_TV", "SB_TV", "TGV", "NDF", "Diff4th", "LLT_ROF", "FGP_dTV", "TV_ENERGY"]


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _prepare(data, gpu_id):
    """Return (input, output, device pointers, dims, stream handle)."""
    if gpu_id < 0:
        raise ValueError("The gpu_device must be a positive integer or zero")
    if _is_torch(data):
        import torch

        if not data.is_cuda:
            raise ValueError("data must be a CUDA tensor")
        if data.dtype != torch.float32:
            raise ValueError("The input data should be float32 data type")
        if data.dim() not in (2, 3):
            raise ValueError("data must be 2D or 3D")
        if data.device.index != gpu_id:
            raise ValueError(f"data is on cuda:{data.device.index}, gpu_id={gpu_id}")
        data = data.contiguous()
        out = torch.empty_like(data)
        stream = torch.cuda.current_stream(data.device).cuda_stream
        shape = tuple(data.shape)
        return data, out, data.data_ptr(), out.data_ptr(), shape, stream
    cai = getattr(data, "__cuda_array_interface__", None)
    if cai is None:
        raise TypeError("data must be a CuPy array, a torch CUDA tensor or expose __cuda_array_interface__")
    if np.dtype(cai["typestr"]) != np.float32:
        raise ValueError("The input data should be float32 data type")
    shape = tuple(cai["shape"])
    if len(shape) not in (2, 3):
        raise ValueError("data must be 2D or 3D")
    if cai.get("strides") not in (None, tuple(np.empty(shape, np.float32).strides)):
        raise ValueError("data must be C-contiguous")
    import cupy as cp  # only CuPy is expected to get here

    cp.cuda.Device(gpu_id).use()
    out = cp.empty(shape, dtype=cp.float32)
    stream = cp.cuda.get_current_stream().ptr
    return data, out, int(cai["data"][0]), out.data.ptr, shape, stream


def _dims(shape):
    d = list(shape)[::-1]
    if len(shape) == 2:
        d.append(1)
    return d


def _info(infovector):
    if infovector is None:
        return np.zeros(2, np.float32)
    if infovector.dtype != np.float32 or infovector.size < 2:
        raise TypeError("infovector must be float32 with at least 2 elements")
    return infovector


def _call(fn, data, gpu_id, infovector, *params):
    data, out, pin, pout, shape, stream = _prepare(data, gpu_id)
    info = _info(infovector)
    st = fn(pin, pout, info.ctypes.data_as(fn.argtypes[2]), *params, *_dims(shape), stream)
    check_status(st)
    return out


def ROF_TV(data, regularisation_parameter=1e-05, iterations=3000, time_marching_parameter=0.001, gpu_id=0,
           tolerance_param=0.0, infovector=None):
    """ROF-TV explicit gradient flow on a device array."""
    return _call(cilregcuda.cilreg_rof_tv_dev, data, gpu_id, infovector, None, float(regularisation_parameter),
                 int(iterations), float(time_marching_parameter), float(tolerance_param))


def PD_TV(data, regularisation_parameter=1e-05, iterations=1000, tolerance_param=0.0, methodTV=0, nonneg=0,
          lipschitz_const=8.0, gpu_id=0, infovector=None):
    """Primal-dual TV on a device array."""
    return _call(cilregcuda.cilreg_pd_tv_dev, data, gpu_id, infovector, float(regularisation_parameter),
                 int(iterations), float(tolerance_param), float(lipschitz_const), int(methodTV), int(nonneg))


def FGP_TV(data, regularisation_parameter=1e-05, iterations=500, tolerance_param=0.0, methodTV=0, nonneg=0,
           gpu_id=0, infovector=None):
    """FGP-TV on a device array (U_prev of iteration 0 is zero)."""
    data, out, pin, pout, shape, stream = _prepare(data, gpu_id)
    # the output starts at zero, as np.zeros_like in the reference's TV.py:76
    if _is_torch(out):
        out.zero_()
    else:
        out.fill(0)
    info = _info(infovector)
    fn = cilregcuda.cilreg_fgp_tv_dev
    st = fn(pin, pout, info.ctypes.data_as(fn.argtypes[2]), float(regularisation_parameter), int(iterations),
            float(tolerance_param), int(methodTV), int(nonneg), *_dims(shape), stream)
    check_status(st)
    return out


def SB_TV(data, regularisation_parameter=1e-05, iterations=100, tolerance_param=0.0, methodTV=0, gpu_id=0,
          infovector=None):
    """Split-Bregman TV on a device array (regularisation_parameter is the reference's mu)."""
    return _call(cilregcuda.cilreg_sb_tv_dev, data, gpu_id, infovector, float(regularisation_parameter),
                 int(iterations), float(tolerance_param), int(methodTV))


def TGV(data, regularisation_parameter=1e-05, alpha1=1.0, alpha0=2.0, iterations=500, lipschitz_const=12.0,
        tolerance_param=0.0, gpu_id=0, infovector=None):
    """TGV^2 on a device array."""
    return _call(cilregcuda.cilreg_tgv_dev, data, gpu_id, infovector, float(regularisation_parameter),
                 float(alpha1), float(alpha0), int(iterations), float(lipschitz_const), float(tolerance_param))


def NDF(data, regularisation_parameter=1e-05, edge_parameter=0.01, iterations=500, time_marching_parameter=0.01,
        penalty_type=1, tolerance_param=0.0, gpu_id=0, infovector=None):
    """Non-linear diffusion (Jacobi order) on a device array."""
    return _call(cilregcuda.cilreg_ndf_dev, data, gpu_id, infovector, float(regularisation_parameter),
                 float(edge_parameter), int(iterations), float(time_marching_parameter), int(penalty_type),
                 float(tolerance_param))


def Diff4th(data, regularisation_parameter=1e-05, edge_parameter=0.01, iterations=500,
            time_marching_parameter=0.0001, tolerance_param=0.0, gpu_id=0, infovector=None):
    """Fourth-order diffusion on a device array."""
    return _call(cilregcuda.cilreg_diff4th_dev, data, gpu_id, infovector, float(regularisation_parameter),
                 float(edge_parameter), int(iterations), float(time_marching_parameter), float(tolerance_param))


def LLT_ROF(data, regularisation_parameterROF=1e-05, regularisation_parameterLLT=1e-05, iterations=500,
            time_marching_parameter=0.0001, tolerance_param=0.0, gpu_id=0, infovector=None):
    """LLT-ROF on a device array."""
    return _call(cilregcuda.cilreg_llt_rof_dev, data, gpu_id, infovector, float(regularisation_parameterROF),
                 float(regularisation_parameterLLT), int(iterations), float(time_marching_parameter),
                 float(tolerance_param))


def _pointer_like(ref, data, shape):
    """Device pointer of `ref`, which must match data's kind, shape and dtype."""
    if _is_torch(data):
        if not _is_torch(ref) or tuple(ref.shape) != shape or ref.dtype != data.dtype or ref.device != data.device:
            raise ValueError("refdata must be a float32 CUDA tensor of the input's shape and device")
        ref = ref.contiguous()
        return ref, ref.data_ptr()
    cai = getattr(ref, "__cuda_array_interface__", None)
    if cai is None or tuple(cai["shape"]) != shape or np.dtype(cai["typestr"]) != np.float32:
        raise ValueError("refdata must be a float32 device array of the input's shape")
    return ref, int(cai["data"][0])


def FGP_dTV(data, refdata, regularisation_parameter=1e-05, iterations=500, tolerance_param=0.0, eta_const=0.01,
            methodTV=0, nonneg=0, gpu_id=0, infovector=None):
    """FGP-dTV on device arrays (U_prev of iteration 0 is zero)."""
    data, out, pin, pout, shape, stream = _prepare(data, gpu_id)
    refdata, pref = _pointer_like(refdata, data, shape)
    if _is_torch(out):
        out.zero_()
    else:
        out.fill(0)
    info = _info(infovector)
    fn = cilregcuda.cilreg_dtv_fgp_dev
    st = fn(pin, pref, pout, info.ctypes.data_as(fn.argtypes[3]), float(regularisation_parameter), int(iterations),
            float(tolerance_param), float(eta_const), int(methodTV), int(nonneg), *_dims(shape), stream)
    check_status(st)
    return out


def TV_ENERGY(data, data0, regularisation_parameter, type=1, gpu_id=0):
    """TV energy of device arrays (type 1: 2 lambda TV + |u - u0|^2; type 2: 2 lambda TV); a float."""
    data, _, pin, _, shape, stream = _prepare(data, gpu_id)
    data0, p0 = _pointer_like(data0, data, shape)
    e = np.zeros(1, np.float32)
    fn = cilregcuda.cilreg_tv_energy_dev
    st = fn(pin, p0, e.ctypes.data_as(fn.argtypes[2]), float(regularisation_parameter), int(type), *_dims(shape),
            stream)
    check_status(st)
    return float(e[0])
