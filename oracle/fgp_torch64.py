"""ORACLE — TEST INFRASTRUCTURE ONLY.

The unrolled FGP-TV map in FP64 torch (CPU), written with differentiable
torch operations so that torch's own autograd provides an independent
gradient to check the library's hand-written adjoint against.  It restates
FGP_TV_core.c:40-269 with the projection of utils.c:149-213 (no stopping
rule); the momentum sequence t_k is formed in float32 exactly as the
reference does (FGP_TV_core.c:138), so both sides use identical coefficients.
Arrays are (Z, Y, X) or (Y, X); component 0 is the x (fastest) axis.
"""
from __future__ import annotations

import numpy as np
import torch


def _shift_back(x, dim):
    """x[i-1] along dim, 0 at i = 0 (the R[-1] = 0 boundary of Obj_func)."""
    zero = torch.zeros_like(x.narrow(dim, 0, 1))
    return torch.cat([zero, x.narrow(dim, 0, x.shape[dim] - 1)], dim=dim)


def _fwd_diff(u, dim):
    """u[i] - u[i+1] along dim, 0 at the last index (Grad_func)."""
    zero = torch.zeros_like(u.narrow(dim, 0, 1))
    n = u.shape[dim]
    return torch.cat([u.narrow(dim, 0, n - 1) - u.narrow(dim, 1, n - 1), zero], dim=dim)


def momentum(iters: int):
    """cc[k]: coefficient iteration k uses to form R_k (cc[0] = 0), float32 like the reference."""
    tk = np.float32(1.0)
    cprev = np.float32(0.0)
    out = []
    for _ in range(iters):
        out.append(float(cprev))
        tkp1 = np.float32((np.float32(1.0) + np.sqrt(np.float32(1.0) + np.float32(4.0) * tk * tk)) * np.float32(0.5))
        cprev = np.float32((tk - np.float32(1.0)) / tkp1)
        tk = tkp1
    return out


def fgp_unrolled(f: torch.Tensor, lam: torch.Tensor, iters: int, method: int = 0, nonneg: int = 0):
    three = f.dim() == 3
    dims = [-1, -2, -3] if three else [-1, -2]
    m = 1.0 / (12.0 * lam) if three else 1.0 / (8.0 * lam)
    zero = torch.zeros_like(f)
    P = [zero for _ in dims]
    Pold = [zero for _ in dims]
    u = f
    for k, c in enumerate(momentum(iters)):
        R = [p + c * (p - q) for p, q in zip(P, Pold)]
        div = sum(r - _shift_back(r, dd) for r, dd in zip(R, dims))
        u = f - lam * div
        if nonneg:
            u = torch.clamp(u, min=0.0)
        if k == iters - 1:
            break
        Q = [r + m * _fwd_diff(u, dd) for r, dd in zip(R, dims)]
        if method == 0:
            den = sum(q * q for q in Q)
            scale = torch.where(den > 1.0, 1.0 / torch.sqrt(torch.clamp(den, min=1.0)), torch.ones_like(den))
            Pn = [q * scale for q in Q]
        else:
            Pn = [q / torch.clamp(torch.abs(q), min=1.0) for q in Q]
        Pold, P = P, Pn
    return u
