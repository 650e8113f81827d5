"""Argument marshalling shared by TV.py and diffusion.py.

The reference passes ``ndarray.ctypes`` pointers without checking dtype or
layout (src/Python/ccpi/filters/TV.py:25-42), so a float64 or strided array
is silently misread.  Here inputs must be float32 ndarrays of 2 or 3
dimensions; non-contiguous inputs are copied, and ``out`` / ``infovector``
are validated before any native call.
"""
from __future__ import annotations

import ctypes

import numpy as np

_P = ctypes.POINTER(ctypes.c_float)


def as_input(a) -> np.ndarray:
    if not isinstance(a, np.ndarray):
        raise TypeError(f"inputData must be a numpy.ndarray, got {type(a).__name__}")
    if a.dtype != np.float32:
        raise TypeError(f"inputData must be float32, got {a.dtype}")
    if a.ndim not in (2, 3):
        raise ValueError(f"inputData must be 2D or 3D, got shape {a.shape}")
    if a.size == 0:
        raise ValueError("inputData is empty")
    return np.ascontiguousarray(a)


def as_output(out, like: np.ndarray, zero_init: bool = True) -> np.ndarray:
    """The caller's output array, validated, or a new one.  The GPU entry
    points write their Output whole (they never read it unless they run no
    iteration), so their wrappers ask for no zero fill: a 512 MiB np.zeros_like
    costs tens of milliseconds per call."""
    if out is None:
        return np.zeros_like(like) if zero_init else np.empty_like(like)
    if not isinstance(out, np.ndarray) or out.dtype != np.float32:
        raise TypeError("out must be a float32 numpy.ndarray")
    if out.shape != like.shape:
        raise ValueError(f"out has shape {out.shape}, expected {like.shape}")
    if not out.flags.c_contiguous or not out.flags.writeable:
        raise ValueError("out must be C-contiguous and writeable")
    return out


def as_info(infovector) -> np.ndarray:
    if infovector is None:
        return np.zeros((2,), dtype=np.float32)
    if (not isinstance(infovector, np.ndarray) or infovector.dtype != np.float32 or infovector.size < 2
            or not infovector.flags.c_contiguous):
        raise TypeError("infovector must be a contiguous float32 ndarray with at least 2 elements")
    return infovector


def dims(a: np.ndarray):
    """(dimX, dimY, dimZ) with dimX the fastest axis, as TV.py:37-39."""
    d = list(a.shape)[::-1]
    if a.ndim == 2:
        d.append(1)
    return d


def ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)
