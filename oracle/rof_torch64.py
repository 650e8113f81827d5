"""ORACLE — TEST INFRASTRUCTURE ONLY.

The unrolled ROF-TV map in FP64 torch (CPU), written with differentiable
torch operations so that torch's own autograd provides an independent
gradient to check the library's hand-written ROF adjoint against.  It
restates ROF_TV_core.c:50-317 (scalar lambda, no stopping rule): the fluxes
D1 (j axis), D2 (i axis), D3 (k axis) of D1_func/D2_func/D3_func
(:102-266) with their symmetric (mirrored) boundaries and the update of
TV_kernel (:269-317).  Arrays are (Z, Y, X) or (Y, X).
"""
from __future__ import annotations

import numpy as np
import torch


def _mirror(n: int, shift: int) -> torch.Tensor:
    """Neighbour index i + shift with the reference's reflection
    (i1 = i + 1 -> i - 1 past the end, i2 = i - 1 -> i + 1 before the start);
    an axis of length 1 maps to itself."""
    if n == 1:
        return torch.zeros(1, dtype=torch.long)
    idx = np.arange(n) + shift
    idx[idx >= n] = n - 2
    idx[idx < 0] = 1
    return torch.tensor(idx, dtype=torch.long)


def _minmod(a, b):
    return 0.5 * (torch.sign(a) + torch.sign(b)) * torch.minimum(a.abs(), b.abs())


def rof_step(u: torch.Tensor, f: torch.Tensor, lam, tau: float) -> torch.Tensor:
    """One iteration: fluxes of D1_func/D2_func/D3_func, update of TV_kernel."""
    dims = [-1, -2, -3] if u.dim() == 3 else [-1, -2]
    hi = [_mirror(u.shape[d], 1) for d in dims]
    lo = [_mirror(u.shape[d], -1) for d in dims]
    fwd = [u.index_select(d, h) - u for d, h in zip(dims, hi)]
    bwd = [u - u.index_select(d, l) for d, l in zip(dims, lo)]
    mm = [_minmod(p, q) for p, q in zip(fwd, bwd)]
    div = 0.0
    for a, (d, l) in enumerate(zip(dims, lo)):
        s = fwd[a] * fwd[a] + 1.0e-8
        for b in range(len(dims)):
            if b != a:
                s = s + mm[b] * mm[b]
        flux = fwd[a] / torch.sqrt(s)
        div = div + flux - flux.index_select(d, l)
    return u + tau * (lam * div - (u - f))


def rof_unrolled(f: torch.Tensor, lam: torch.Tensor, iters: int, tau: float) -> torch.Tensor:
    u = f
    for _ in range(iters):
        u = rof_step(u, f, lam, tau)
    return u
