"""Seeded piecewise-constant phantoms used as synthetic workloads.

A "painter's" phantom on the normalised grid [-1, 1]^d: for each shape, drawn
from ``numpy.random.default_rng(seed)``,

* centre ~ U[-0.7, 0.7]^d, semi-axes ~ U[0.05, 0.5]^d,
* one rotation angle ~ U[0, pi) in 2D, three Euler angles ~ U[0, pi) in 3D,
* intensity ~ U[0, 1];

later shapes overwrite earlier ones, the background is 0, and i.i.d.
N(0, noise^2) noise is added before the cast to float32.  Each shape is
rasterised inside its bounding box only, so a 512^3 volume takes seconds.
"""
from __future__ import annotations

import numpy as np


def _axis(n: int) -> np.ndarray:
    # cell-centred coordinates on [-1, 1]
    return ((np.arange(n, dtype=np.float64) + 0.5) / n) * 2.0 - 1.0


def _rot3(a: float, b: float, c: float) -> np.ndarray:
    ca, sa, cb, sb, cc, sc = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(c), np.sin(c)
    rz1 = np.array([[ca, -sa, 0.0], [sa, ca, 0.0], [0.0, 0.0, 1.0]])
    rx = np.array([[1.0, 0.0, 0.0], [0.0, cb, -sb], [0.0, sb, cb]])
    rz2 = np.array([[cc, -sc, 0.0], [sc, cc, 0.0], [0.0, 0.0, 1.0]])
    return rz1 @ rx @ rz2


def _window(axis: np.ndarray, lo: float, hi: float) -> slice:
    i0 = int(np.searchsorted(axis, lo, side="left"))
    i1 = int(np.searchsorted(axis, hi, side="right"))
    return slice(i0, i1)


def clean_phantom(shape, n_shapes: int, seed: int) -> np.ndarray:
    """Noise-free phantom of ``shape`` ((Y, X) or (Z, Y, X)), float32."""
    shape = tuple(int(s) for s in shape)
    rng = np.random.default_rng(seed)
    d = len(shape)
    if d not in (2, 3):
        raise ValueError("shape must be 2D or 3D")
    img = np.zeros(shape, dtype=np.float32)
    axes = [_axis(n) for n in shape]  # axes[0] is the slowest (Z or Y)
    for _ in range(n_shapes):
        centre = rng.uniform(-0.7, 0.7, size=d)
        semi = rng.uniform(0.05, 0.5, size=d)
        if d == 2:
            th = rng.uniform(0.0, np.pi)
            rot = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
        else:
            rot = _rot3(*rng.uniform(0.0, np.pi, size=3))
        value = np.float32(rng.uniform(0.0, 1.0))
        # bounding box of the rotated ellipse(oid): half-width along axis a is
        # sqrt(sum_b (R[a,b] * semi[b])^2)
        half = np.sqrt(((rot * semi[None, :]) ** 2).sum(axis=1))
        win = tuple(_window(axes[a], centre[a] - half[a], centre[a] + half[a]) for a in range(d))
        if any(w.stop <= w.start for w in win):
            continue
        grids = np.meshgrid(*[axes[a][win[a]] - centre[a] for a in range(d)], indexing="ij")
        # body-frame coordinates q = R^T (x - c)
        q = [sum(rot[a, b] * grids[a] for a in range(d)) for b in range(d)]
        inside = sum((q[b] / semi[b]) ** 2 for b in range(d)) <= 1.0
        img[win][inside] = value
    return img


def noisy_phantom(shape, n_shapes: int, seed: int, noise: float = 0.05) -> np.ndarray:
    """Phantom plus i.i.d. Gaussian noise of standard deviation ``noise`` (float32)."""
    img = clean_phantom(shape, n_shapes, seed)
    rng = np.random.default_rng(seed + 1_000_003)
    out = img
    # add noise in slabs to bound temporary memory on large volumes
    flat = out.reshape(-1)
    step = 1 << 24
    for s in range(0, flat.size, step):
        e = min(flat.size, s + step)
        flat[s:e] += rng.normal(0.0, noise, size=e - s).astype(np.float32)
    return out
