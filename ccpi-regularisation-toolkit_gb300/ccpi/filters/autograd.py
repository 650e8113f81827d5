"""Differentiable FGP-TV and ROF-TV for torch: ``fgp_tv(f, lam, iterations)``
and ``rof_tv(f, lam, iterations, tau)``.

The forward pass is the production GPU iteration (no stopping rule); the
backward pass is the library's hand-written adjoint of the unrolled
iterations (``cilreg_fgp_tv_vjp_dev`` / ``cilreg_rof_tv_vjp_dev``), which
stores the forward states every ``checkpoint`` iterations and recomputes each
segment before its reverse sweep.  Gradients flow to the input volume(s) and
to the regularisation parameter, so lambda can be learned.

``f`` is a float32 CUDA tensor of shape (Y, X), (Z, Y, X) or a batch
(B, Z, Y, X) / (B, Y, X) when ``batched=True``; ``lam`` is a float or a
0-d / (B,) tensor.
"""
from __future__ import annotations

import ctypes
from concurrent.futures import ThreadPoolExecutor

import torch

from .utils import check_status, cilregcuda


def _dims(shape):
    d = list(shape)[::-1]
    if len(shape) == 2:
        d.append(1)
    return d


def _forward_one(f, lam, iters, method, nonneg):
    out = torch.zeros_like(f)
    info = (ctypes.c_float * 2)()
    st = cilregcuda.cilreg_fgp_tv_dev(f.data_ptr(), out.data_ptr(), info, float(lam), int(iters), 0.0, int(method),
                                      int(nonneg), *_dims(tuple(f.shape)),
                                      torch.cuda.current_stream(f.device).cuda_stream)
    check_status(st)
    return out


def _vjp_one(f, ybar, lam, iters, method, nonneg, ckpt, fbar):
    lb = ctypes.c_double(0.0)
    st = cilregcuda.cilreg_fgp_tv_vjp_dev(f.data_ptr(), ybar.data_ptr(), fbar.data_ptr(), ctypes.byref(lb),
                                          float(lam), int(iters), int(method), int(nonneg), int(ckpt),
                                          *_dims(tuple(f.shape)), torch.cuda.current_stream(f.device).cuda_stream)
    check_status(st)
    return lb.value


def _parallel(vjp, vols, ybars, lams):
    """Run one vector-Jacobian product per volume, concurrently: each volume on
    its own host thread and CUDA stream (the library call releases the GIL and
    returns once its stream is done), so small volumes fill the GPU together.
    Outputs are allocated on the caller's stream before the workers start."""
    fbars = [torch.empty_like(v) for v in vols]
    if len(vols) == 1:
        return fbars, [vjp(vols[0], ybars[0], lams[0], fbars[0])]
    caller = torch.cuda.current_stream(vols[0].device)
    ready = torch.cuda.Event()
    ready.record(caller)

    def work(i):
        s = torch.cuda.Stream(device=vols[i].device)
        s.wait_event(ready)
        with torch.cuda.stream(s):
            return vjp(vols[i], ybars[i], lams[i], fbars[i])

    with ThreadPoolExecutor(max_workers=len(vols)) as ex:
        lbars = list(ex.map(work, range(len(vols))))
    return fbars, lbars


class FGPTVFunction(torch.autograd.Function):
    """y = FGP_TV(f, lam) unrolled for a fixed number of iterations."""

    @staticmethod
    def forward(ctx, f, lam, iterations, methodTV, nonneg, checkpoint, batched):
        if not (f.is_cuda and f.dtype == torch.float32):
            raise TypeError("f must be a float32 CUDA tensor")
        f = f.contiguous()
        vols = list(f) if batched else [f]
        lam_t = torch.as_tensor(lam, dtype=torch.float64).reshape(-1)
        lams = lam_t.expand(len(vols)) if lam_t.numel() == 1 else lam_t
        if lams.numel() != len(vols):
            raise ValueError("lam must be a scalar or hold one value per volume")
        if len(vols) > 1 and vols[0].dim() == 3:
            # all volumes in one batched run (one graph launch, bit-equal to
            # single calls, whose kernel family the batch follows); 2D images
            # run one call each
            from .batch import FGP_TV_batch

            outs = FGP_TV_batch(vols, lams.tolist(), iterations, 0.0, methodTV, nonneg, f.device.index or 0)
        else:
            outs = [_forward_one(v, float(l), iterations, methodTV, nonneg) for v, l in zip(vols, lams.tolist())]
        ctx.save_for_backward(f)
        ctx.lams = lams.tolist()
        ctx.lam_shape = torch.as_tensor(lam).shape
        ctx.cfg = (iterations, methodTV, nonneg, checkpoint, batched)
        return torch.stack(outs) if batched else outs[0]

    @staticmethod
    def backward(ctx, ybar):
        (f,) = ctx.saved_tensors
        iterations, method, nonneg, ckpt, batched = ctx.cfg
        ybar = ybar.contiguous()
        vols = list(f) if batched else [f]
        ybars = list(ybar) if batched else [ybar]
        fbars, lbars = _parallel(lambda v, yb, lam, fb: _vjp_one(v, yb, lam, iterations, method, nonneg, ckpt, fb),
                                 vols, ybars, ctx.lams)
        fbar = torch.stack(fbars) if batched else fbars[0]
        if len(ctx.lam_shape) == 0 or (len(lbars) > 1 and int(torch.tensor(ctx.lam_shape).prod()) == 1):
            lam_bar = torch.tensor(sum(lbars), dtype=torch.float64).reshape(ctx.lam_shape)
        else:
            lam_bar = torch.tensor(lbars, dtype=torch.float64).reshape(ctx.lam_shape)
        return fbar, lam_bar, None, None, None, None, None


def fgp_tv(f, lam, iterations, methodTV=0, nonneg=0, checkpoint=20, batched=False):
    """Differentiable unrolled FGP-TV (gradients w.r.t. ``f`` and ``lam``)."""
    if not torch.is_tensor(lam):
        lam = torch.tensor(float(lam), dtype=torch.float64)
    return FGPTVFunction.apply(f, lam, int(iterations), int(methodTV), int(nonneg), int(checkpoint), bool(batched))


def _rof_forward_one(f, lam, iters, tau):
    out = torch.empty_like(f)
    info = (ctypes.c_float * 2)()
    st = cilregcuda.cilreg_rof_tv_dev(f.data_ptr(), out.data_ptr(), info, None, float(lam), int(iters), float(tau),
                                      0.0, *_dims(tuple(f.shape)), torch.cuda.current_stream(f.device).cuda_stream)
    check_status(st)
    return out


def _rof_vjp_one(f, ybar, lam, iters, tau, ckpt, fbar):
    lb = ctypes.c_double(0.0)
    st = cilregcuda.cilreg_rof_tv_vjp_dev(f.data_ptr(), ybar.data_ptr(), fbar.data_ptr(), ctypes.byref(lb),
                                          float(lam), int(iters), float(tau), int(ckpt), *_dims(tuple(f.shape)),
                                          torch.cuda.current_stream(f.device).cuda_stream)
    check_status(st)
    return lb.value


def _per_volume_lams(lam, nvol):
    lam_t = torch.as_tensor(lam, dtype=torch.float64).reshape(-1)
    lams = lam_t.expand(nvol) if lam_t.numel() == 1 else lam_t
    if lams.numel() != nvol:
        raise ValueError("lam must be a scalar or hold one value per volume")
    return lams.tolist()


def _lam_grad(lbars, lam_shape):
    if len(lam_shape) == 0 or (len(lbars) > 1 and int(torch.tensor(lam_shape).prod()) == 1):
        return torch.tensor(sum(lbars), dtype=torch.float64).reshape(lam_shape)
    return torch.tensor(lbars, dtype=torch.float64).reshape(lam_shape)


class ROFTVFunction(torch.autograd.Function):
    """y = ROF_TV(f, lam) unrolled for a fixed number of iterations (scalar lambda per volume)."""

    @staticmethod
    def forward(ctx, f, lam, iterations, tau, checkpoint, batched):
        if not (f.is_cuda and f.dtype == torch.float32):
            raise TypeError("f must be a float32 CUDA tensor")
        f = f.contiguous()
        vols = list(f) if batched else [f]
        lams = _per_volume_lams(lam, len(vols))
        outs = [_rof_forward_one(v, l, iterations, tau) for v, l in zip(vols, lams)]
        ctx.save_for_backward(f)
        ctx.lams = lams
        ctx.lam_shape = torch.as_tensor(lam).shape
        ctx.cfg = (iterations, tau, checkpoint, batched)
        return torch.stack(outs) if batched else outs[0]

    @staticmethod
    def backward(ctx, ybar):
        (f,) = ctx.saved_tensors
        iterations, tau, ckpt, batched = ctx.cfg
        ybar = ybar.contiguous()
        vols = list(f) if batched else [f]
        ybars = list(ybar) if batched else [ybar]
        fbars, lbars = _parallel(lambda v, yb, lam, fb: _rof_vjp_one(v, yb, lam, iterations, tau, ckpt, fb),
                                 vols, ybars, ctx.lams)
        fbar = torch.stack(fbars) if batched else fbars[0]
        return fbar, _lam_grad(lbars, ctx.lam_shape), None, None, None, None


def rof_tv(f, lam, iterations, tau, checkpoint=20, batched=False):
    """Differentiable unrolled ROF-TV (gradients w.r.t. ``f`` and ``lam``)."""
    if not torch.is_tensor(lam):
        lam = torch.tensor(float(lam), dtype=torch.float64)
    return ROFTVFunction.apply(f, lam, int(iterations), float(tau), int(checkpoint), bool(batched))
