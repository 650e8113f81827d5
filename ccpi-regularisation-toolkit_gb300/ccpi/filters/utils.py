"""Loads the GB300 regulariser libraries (the reference's
src/Python/ccpi/filters/utils.py:13-23 loads ``libcilreg`` and
``libcilregcuda`` from this directory the same way).

Both libraries are required: there is no CPU fallback.  If they are missing,
build them with ``python build.py`` in the package root.  ``libcilreg.so``
forwards every entry point to ``libcilregcuda.so``, so the process holds one
copy of the GPU library whichever name a caller binds.
"""
import ctypes
import os
import platform

if platform.system() != "Linux":
    raise ImportError(f"unsupported platform: {platform.system()} (this build targets Linux on GB300)")

_here = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_here, "libcilreg.so")
GPU_LIB_PATH = os.path.join(_here, "libcilregcuda.so")

for _p in (LIB_PATH, GPU_LIB_PATH):
    if not os.path.exists(_p):
        raise ImportError(f"{_p} is not built; run `python build.py` in "
                          f"{os.path.dirname(os.path.dirname(_here))}")

cilreg = ctypes.CDLL(LIB_PATH)
cilregcuda = ctypes.CDLL(GPU_LIB_PATH)

_F = ctypes.c_float
_I = ctypes.c_int
_P = ctypes.POINTER(ctypes.c_float)
_V = ctypes.c_void_p

# *_CPU_main argument lists (src/Core/regularisers_CPU/*_core.h)
_CPU_SIGS = {
    "TV_ROF_CPU_main": [_P, _P, _P, _P, _I, _I, _F, _F, _I, _I, _I],
    "TV_FGP_CPU_main": [_P, _P, _P, _F, _I, _F, _I, _I, _I, _I, _I],
    "PDTV_CPU_main": [_P, _P, _P, _F, _I, _F, _F, _I, _I, _I, _I, _I],
    "SB_TV_CPU_main": [_P, _P, _P, _F, _I, _F, _I, _I, _I, _I],
    "TGV_main": [_P, _P, _P, _F, _F, _F, _I, _F, _F, _I, _I, _I],
    "Diffusion_CPU_main": [_P, _P, _P, _F, _F, _I, _F, _I, _F, _I, _I, _I],
    "Diffus4th_CPU_main": [_P, _P, _P, _F, _F, _I, _F, _F, _I, _I, _I],
    "LLT_ROF_CPU_main": [_P, _P, _P, _F, _F, _I, _F, _F, _I, _I, _I],
    "dTV_FGP_CPU_main": [_P, _P, _P, _P, _F, _I, _F, _F, _I, _I, _I, _I, _I],
    "TV_energy2D": [_P, _P, _P, _F, _I, _I, _I],
    "TV_energy3D": [_P, _P, _P, _F, _I, _I, _I, _I],
}
# *_GPU_main argument lists (src/Core/regularisers_GPU/*.h)
_GPU_SIGS = {
    "TV_ROF_GPU_main": [_P, _P, _P, _F, _I, _F, _F, _I, _I, _I, _I],
    "TV_FGP_GPU_main": [_P, _P, _P, _F, _I, _F, _I, _I, _I, _I, _I, _I],
    "TV_PD_GPU_main": [_P, _P, _P, _F, _I, _F, _F, _I, _I, _I, _I, _I, _I],
    "TV_SB_GPU_main": [_P, _P, _P, _F, _I, _F, _I, _I, _I, _I, _I],
    "TGV_GPU_main": [_P, _P, _P, _F, _F, _F, _I, _F, _F, _I, _I, _I, _I],
    "NonlDiff_GPU_main": [_P, _P, _P, _F, _F, _I, _F, _I, _F, _I, _I, _I, _I],
    "Diffus4th_GPU_main": [_P, _P, _P, _F, _F, _I, _F, _F, _I, _I, _I, _I],
    "LLT_ROF_GPU_main": [_P, _P, _P, _F, _F, _I, _F, _F, _I, _I, _I, _I],
    "dTV_FGP_GPU_main": [_P, _P, _P, _P, _F, _I, _F, _F, _I, _I, _I, _I, _I, _I],
}
# device-pointer API (include/cilreg_gb300.h)
_DEV_SIGS = {
    "cilreg_rof_tv_dev": [_V, _V, _P, _V, _F, _I, _F, _F, _I, _I, _I, _V],
    "cilreg_fgp_tv_dev": [_V, _V, _P, _F, _I, _F, _I, _I, _I, _I, _I, _V],
    "cilreg_pd_tv_dev": [_V, _V, _P, _F, _I, _F, _F, _I, _I, _I, _I, _I, _V],
    "cilreg_sb_tv_dev": [_V, _V, _P, _F, _I, _F, _I, _I, _I, _I, _V],
    "cilreg_tgv_dev": [_V, _V, _P, _F, _F, _F, _I, _F, _F, _I, _I, _I, _V],
    "cilreg_ndf_dev": [_V, _V, _P, _F, _F, _I, _F, _I, _F, _I, _I, _I, _V],
    "cilreg_diff4th_dev": [_V, _V, _P, _F, _F, _I, _F, _F, _I, _I, _I, _V],
    "cilreg_llt_rof_dev": [_V, _V, _P, _F, _F, _I, _F, _F, _I, _I, _I, _V],
    "cilreg_dtv_fgp_dev": [_V, _V, _V, _P, _F, _I, _F, _F, _I, _I, _I, _I, _I, _V],
    "cilreg_tv_energy_dev": [_V, _V, _P, _F, _I, _I, _I, _I, _V],
}

_PP = ctypes.POINTER(ctypes.c_void_p)
_IP = ctypes.POINTER(ctypes.c_int)
_VJP_SIGS = {
    "cilreg_fgp_tv_vjp_dev": [_V, _V, _V, ctypes.POINTER(ctypes.c_double), _F, _I, _I, _I, _I, _I, _I, _I, _V],
    "cilreg_rof_tv_vjp_dev": [_V, _V, _V, ctypes.POINTER(ctypes.c_double), _F, _I, _F, _I, _I, _I, _I, _V],
}
_SESSION_SIGS = {
    "cilreg_prox_session_create": [ctypes.POINTER(ctypes.c_void_p), _I, _P, _I, _I, _I, _I, _V],
    "cilreg_prox_session_prox": [_V, _V, _V, _I, _F, _P, _V],
    "cilreg_prox_session_fista": [_V, _V, _V, _I, _I, _F, _V],
    "cilreg_prox_session_admm": [_V, _V, _V, _V, _I, _I, _F, _V],
    "cilreg_prox_session_pdhg": [_V, _V, _V, _V, _I, _I, _F, _F, _V],
    "cilreg_prox_session_set_cancel": [_V, _IP],
    "cilreg_prox_session_destroy": [_V, _V],
    "cilreg_debug_fail_allocations": [_I],
}
_BATCH_SIGS = {
    "cilreg_fgp_tv_batch_dev": [_I, _PP, _PP, _IP, _P, _I, _F, _I, _I, _P, _V],
    "cilreg_tgv_batch_dev": [_I, _PP, _PP, _IP, _P, _F, _F, _I, _F, _F, _P, _V],
}

for _lib in (cilreg, cilregcuda):
    for _name, _args in _CPU_SIGS.items():
        getattr(_lib, _name).argtypes = _args
        getattr(_lib, _name).restype = ctypes.c_float
    for _name, _args in {**_GPU_SIGS, **_DEV_SIGS, **_BATCH_SIGS, **_VJP_SIGS, **_SESSION_SIGS}.items():
        getattr(_lib, _name).argtypes = _args
        getattr(_lib, _name).restype = ctypes.c_int
    _lib.cilreg_last_error.restype = ctypes.c_char_p
    _lib.cilreg_version.restype = ctypes.c_char_p
    _lib.cilreg_device_count.restype = ctypes.c_int
    _lib.cilreg_launch_count.restype = ctypes.c_longlong
    _lib.cilreg_release_cached.argtypes = [_I]
    _lib.cilreg_release_cached.restype = ctypes.c_int
    _lib.cilreg_prox_session_bytes.argtypes = [_I, _I, _I, _I]
    _lib.cilreg_prox_session_bytes.restype = ctypes.c_longlong


class RegulariserError(RuntimeError):
    """A regulariser call returned a failure status (-1 CUDA, -3 no device,
    -4 out of memory, -5 cancelled)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"status {status}: {message}")
        self.status = status


def check_status(status, lib=None) -> None:
    """Raise for a negative status (ValueError for invalid arguments)."""
    status = int(status)
    if status == 0:
        return
    msg = (lib or cilregcuda).cilreg_last_error().decode(errors="replace")
    if status == -2:
        raise ValueError(msg)
    raise RegulariserError(status, msg)


def version() -> str:
    return cilregcuda.cilreg_version().decode()


def device_count() -> int:
    return int(cilregcuda.cilreg_device_count())


def launch_count() -> int:
    """Kernels launched so far by the library in this process (libcilreg.so
    forwards to libcilregcuda.so, so both names share one counter)."""
    return int(cilregcuda.cilreg_launch_count())


def release_cached(gpu_device: int = 0) -> None:
    """Wait for the device's work and hand back the scratch memory the library
    keeps cached in the device's stream-ordered pool."""
    check_status(cilregcuda.cilreg_release_cached(int(gpu_device)))


def loaded_libraries():
    """Paths of the two native libraries this module loaded."""
    return [LIB_PATH, GPU_LIB_PATH]
