"""Batched regularisation of many volumes of uneven shape in one call.

``FGP_TV_batch`` and ``TGV_batch`` take a list of volumes (torch CUDA tensors,
or float32 numpy arrays which are uploaded and the results downloaded) and
return the list of results.  All volumes advance together on the GPU: one
kernel launch per iteration covers the tiles of every volume and the whole
iteration loop runs as one CUDA graph.  Each volume keeps its own stopping
rule; results equal those of the single-volume calls (``regularisers.FGP_TV``,
``regularisers.TGV``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from .utils import check_status, cilregcuda


def _dims(shape):
    d = list(shape)[::-1]
    if len(shape) == 2:
        d.append(1)
    return d


def _prepare(volumes, gpu_id):
    import torch

    if len(volumes) == 0:
        raise ValueError("empty batch")
    host = not isinstance(volumes[0], torch.Tensor)
    dev = torch.device("cuda", gpu_id)
    ins = []
    for v in volumes:
        if isinstance(v, torch.Tensor):
            if not v.is_cuda or v.dtype != torch.float32 or v.dim() not in (2, 3):
                raise ValueError("volumes must be float32 CUDA tensors of 2 or 3 dimensions")
            ins.append(v.contiguous())
        else:
            a = np.asarray(v)
            if a.dtype != np.float32 or a.ndim not in (2, 3):
                raise TypeError("volumes must be float32 arrays of 2 or 3 dimensions")
            ins.append(torch.from_numpy(np.ascontiguousarray(a)).to(dev))
    outs = [torch.zeros_like(t) for t in ins]
    n = len(ins)
    pin = (ctypes.c_void_p * n)(*[t.data_ptr() for t in ins])
    pout = (ctypes.c_void_p * n)(*[t.data_ptr() for t in outs])
    dims = (ctypes.c_int * (3 * n))(*[x for t in ins for x in _dims(tuple(t.shape))])
    stream = torch.cuda.current_stream(dev).cuda_stream
    return host, ins, outs, pin, pout, dims, stream


def _lams(lam, n):
    arr = np.broadcast_to(np.asarray(lam, dtype=np.float32), (n,)).copy()
    return arr, arr.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _info(infovectors, n):
    if infovectors is None:
        infovectors = np.zeros((n, 2), np.float32)
    if infovectors.dtype != np.float32 or infovectors.size < 2 * n or not infovectors.flags.c_contiguous:
        raise TypeError("infovectors must be a contiguous float32 array of shape (nvol, 2)")
    return infovectors, infovectors.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _finish(host, outs):
    if host:
        return [o.cpu().numpy() for o in outs]
    return outs


def FGP_TV_batch(volumes, lambdaPar, iterationsNumb, epsil=0.0, methodTV=0, nonneg=0, gpu_id=0, infovectors=None):
    """FGP-TV of every volume; lambdaPar is a scalar or one value per volume."""
    host, ins, outs, pin, pout, dims, stream = _prepare(volumes, gpu_id)
    lam, lam_p = _lams(lambdaPar, len(ins))
    info, info_p = _info(infovectors, len(ins))
    st = cilregcuda.cilreg_fgp_tv_batch_dev(len(ins), pin, pout, dims, lam_p, int(iterationsNumb), float(epsil),
                                            int(methodTV), int(nonneg), info_p, stream)
    check_status(st)
    return _finish(host, outs)


def TGV_batch(volumes, lambdaPar, alpha1, alpha0, iterationsNumb, L2, epsil=0.0, gpu_id=0, infovectors=None):
    """TGV of every volume; lambdaPar is a scalar or one value per volume."""
    host, ins, outs, pin, pout, dims, stream = _prepare(volumes, gpu_id)
    lam, lam_p = _lams(lambdaPar, len(ins))
    info, info_p = _info(infovectors, len(ins))
    st = cilregcuda.cilreg_tgv_batch_dev(len(ins), pin, pout, dims, lam_p, float(alpha1), float(alpha0),
                                         int(iterationsNumb), float(L2), float(epsil), info_p, stream)
    check_status(st)
    return _finish(host, outs)
