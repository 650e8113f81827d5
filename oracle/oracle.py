"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes access to the two CPU checkers:

* ``liboracle_port.so`` — the plain-C restatement in ``cilreg_port.c``; built by
  ``make -C oracle`` on any machine (x86-64 here, aarch64 on the GPU host).
* ``_ref/libcilreg_ref.so`` — the reference toolkit's own C-OMP sources,
  compiled by ``make -C oracle ref`` where those sources exist.

Both expose the reference's ``*_CPU_main`` argument lists
(src/Core/regularisers_CPU/*_core.h).  Only tests, the smoke check and the
benchmark's CPU-baseline leg import this module.  Arrays are C-ordered float32
of shape (Z, Y, X) or (Y, X); dimX is the fastest axis, as in
src/Python/ccpi/filters/TV.py:37-39.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(HERE, "liboracle_port.so")
REF_PATH = os.path.join(HERE, "_ref", "libcilreg_ref.so")

_F = ctypes.c_float
_I = ctypes.c_int
_P = ctypes.POINTER(ctypes.c_float)


def build(ref: bool = True) -> None:
    """Compile the port (and the reference, when its sources are present)."""
    subprocess.run(["make", "-s", "-C", HERE, "ref" if ref else "all"], check=True)


def _load(path):
    if not os.path.exists(path):
        return None
    try:
        return ctypes.CDLL(path)
    except OSError:
        return None


_port = None
_ref = None


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_PATH):
            build(ref=False)
        _port = _load(PORT_PATH)
        if _port is None:
            raise RuntimeError(f"cannot load oracle port {PORT_PATH}")
        _declare(_port, prefix="port_")
        _port.port_num_threads.restype = ctypes.c_int
        _port.port_TV_ROF_init.argtypes = [_P, _P, _P, _F, _I, _F, _F, _I, _I, _I, _P]
        _port.port_TV_FGP_warm.argtypes = [_P, _P, _P, _F, _I, _F, _I, _I, _I, _I, _I, _P]
        _port.port_SB_TV_warm.argtypes = [_P, _P, _P, _F, _I, _F, _I, _I, _I, _I, _P]
        _port.port_Diffusion_init.argtypes = [_P, _P, _P, _F, _F, _I, _F, _I, _F, _I, _I, _I, _P]
        for name in ("port_TV_ROF_init", "port_TV_FGP_warm", "port_SB_TV_warm", "port_Diffusion_init"):
            getattr(_port, name).restype = ctypes.c_float
        _port.port_set_trace.argtypes = [_P, ctypes.c_int]
        _port.port_trace_len.restype = ctypes.c_int
    return _port


def ref_lib():
    """The compiled reference C-OMP library, or None when it is not built here."""
    global _ref
    if _ref is None:
        _ref = _load(REF_PATH)
        if _ref is not None:
            _declare(_ref, prefix=None)
    return _ref


_SIGS = {
    # name in reference, name in port, argtypes after (Input, Output, infovector)
    "TV_ROF": ("TV_ROF_CPU_main", "port_TV_ROF", [_P, _I, _I, _F, _F]),
    "TV_FGP": ("TV_FGP_CPU_main", "port_TV_FGP", [_F, _I, _F, _I, _I]),
    "PDTV": ("PDTV_CPU_main", "port_PDTV", [_F, _I, _F, _F, _I, _I]),
    "SB_TV": ("SB_TV_CPU_main", "port_SB_TV", [_F, _I, _F, _I]),
    "TGV": ("TGV_main", "port_TGV", [_F, _F, _F, _I, _F, _F]),
    "Diffusion": ("Diffusion_CPU_main", "port_Diffusion", [_F, _F, _I, _F, _I, _F]),
    "Diffus4th": ("Diffus4th_CPU_main", "port_Diffus4th", [_F, _F, _I, _F, _F]),
    "LLT_ROF": ("LLT_ROF_CPU_main", "port_LLT_ROF", [_F, _F, _I, _F, _F]),
}


def _declare(lib, prefix):
    for key, (refname, portname, extra) in _SIGS.items():
        name = portname if prefix else refname
        fn = getattr(lib, name)
        args = [_P, _P, _P] + extra + [_I, _I, _I]
        if prefix and key == "Diffusion":
            args = args + [_I]  # jacobi flag
        fn.argtypes = args
        fn.restype = ctypes.c_float
    # FGP-dTV: (Input, InputRef, Output, infovector, lambda, iters, epsil, eta, methodTV, nonneg, dims)
    fn = getattr(lib, "port_dTV_FGP" if prefix else "dTV_FGP_CPU_main")
    fn.argtypes = [_P, _P, _P, _P, _F, _I, _F, _F, _I, _I, _I, _I, _I]
    fn.restype = ctypes.c_float
    # TV energy: (U, U0, E_val, lambda, type, dims)
    for nd in (2, 3):
        fn = getattr(lib, (f"port_TV_energy{nd}D" if prefix else f"TV_energy{nd}D"))
        fn.argtypes = [_P, _P, _P, _F, _I] + [_I] * nd
        fn.restype = ctypes.c_float


def _dims(a):
    d = list(a.shape)[::-1]
    if a.ndim == 2:
        d.append(1)
    return d


def _prep(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    out = np.zeros_like(a)
    info = np.zeros(2, dtype=np.float32)
    return a, out, info


def _ptr(a):
    return a.ctypes.data_as(_P)


def _lib(use_ref):
    if use_ref:
        lib = ref_lib()
        if lib is None:
            raise RuntimeError("reference C-OMP library is not built here")
        return lib, False
    return port_lib(), True


def rof_tv(x, lam, iters, tau, epsil, use_ref=False):
    """`lam` is a scalar or a float32 array of x's shape (per-voxel lambda,
    ROF_TV_core.c:280 `lambda_is_arr`)."""
    lib, is_port = _lib(use_ref)
    a, out, info = _prep(x)
    fn = lib.port_TV_ROF if is_port else lib.TV_ROF_CPU_main
    if np.ndim(lam) == 0:
        lam_c = ctypes.c_float(lam)
        fn(_ptr(a), _ptr(out), _ptr(info), ctypes.byref(lam_c), 0, iters, tau, epsil, *_dims(a))
    else:
        lam_a = np.ascontiguousarray(lam, dtype=np.float32)
        assert lam_a.shape == a.shape
        fn(_ptr(a), _ptr(out), _ptr(info), _ptr(lam_a), 1, iters, tau, epsil, *_dims(a))
    return out, info


def fgp_tv(x, lam, iters, epsil, method_tv=0, nonneg=0, use_ref=False):
    lib, is_port = _lib(use_ref)
    a, out, info = _prep(x)
    fn = lib.port_TV_FGP if is_port else lib.TV_FGP_CPU_main
    fn(_ptr(a), _ptr(out), _ptr(info), lam, iters, epsil, method_tv, nonneg, *_dims(a))
    return out, info


def pd_tv(x, lam, iters, epsil, lipschitz=8.0, method_tv=0, nonneg=0, use_ref=False):
    lib, is_port = _lib(use_ref)
    a, out, info = _prep(x)
    fn = lib.port_PDTV if is_port else lib.PDTV_CPU_main
    fn(_ptr(a), _ptr(out), _ptr(info), lam, iters, epsil, lipschitz, method_tv, nonneg, *_dims(a))
    return out, info


def sb_tv(x, mu, iters, epsil, method_tv=0, use_ref=False):
    lib, is_port = _lib(use_ref)
    a, out, info = _prep(x)
    fn = lib.port_SB_TV if is_port else lib.SB_TV_CPU_main
    fn(_ptr(a), _ptr(out), _ptr(info), mu, iters, epsil, method_tv, *_dims(a))
    return out, info


def tgv(x, lam, alpha1, alpha0, iters, L2, epsil, use_ref=False):
    lib, is_port = _lib(use_ref)
    a, out, info = _prep(x)
    fn = lib.port_TGV if is_port else lib.TGV_main
    fn(_ptr(a), _ptr(out), _ptr(info), lam, alpha1, alpha0, iters, L2, epsil, *_dims(a))
    return out, info


def ndf(x, lam, sigma, iters, tau, penalty, epsil, jacobi=True, use_ref=False):
    """Non-linear diffusion.  The port runs Jacobi sweeps (jacobi=True) or the
    reference's in-place lexicographic sweep (jacobi=False, single thread)."""
    lib, is_port = _lib(use_ref)
    a, out, info = _prep(x)
    if is_port:
        lib.port_Diffusion(_ptr(a), _ptr(out), _ptr(info), lam, sigma, iters, tau, penalty, epsil, *_dims(a),
                           1 if jacobi else 0)
    else:
        lib.Diffusion_CPU_main(_ptr(a), _ptr(out), _ptr(info), lam, sigma, iters, tau, penalty, epsil, *_dims(a))
    return out, info


def diff4th(x, lam, sigma, iters, tau, epsil, use_ref=False):
    lib, is_port = _lib(use_ref)
    a, out, info = _prep(x)
    fn = lib.port_Diffus4th if is_port else lib.Diffus4th_CPU_main
    fn(_ptr(a), _ptr(out), _ptr(info), lam, sigma, iters, tau, epsil, *_dims(a))
    return out, info


def llt_rof(x, lam_rof, lam_llt, iters, tau, epsil, use_ref=False):
    """LLT-ROF (LLT_ROF_core.c:54)."""
    lib, is_port = _lib(use_ref)
    a, out, info = _prep(x)
    fn = lib.port_LLT_ROF if is_port else lib.LLT_ROF_CPU_main
    fn(_ptr(a), _ptr(out), _ptr(info), lam_rof, lam_llt, iters, tau, epsil, *_dims(a))
    return out, info


def dtv_fgp(x, ref, lam, iters, epsil, eta, method_tv=0, nonneg=0, use_ref=False):
    """FGP-dTV (FGP_dTV_core.c:46): `ref` is the reference image of x's shape."""
    lib, is_port = _lib(use_ref)
    a, out, info = _prep(x)
    r = np.ascontiguousarray(ref, dtype=np.float32)
    assert r.shape == a.shape
    fn = lib.port_dTV_FGP if is_port else lib.dTV_FGP_CPU_main
    fn(_ptr(a), _ptr(r), _ptr(out), _ptr(info), lam, iters, epsil, eta, method_tv, nonneg, *_dims(a))
    return out, info


def tv_energy(u, u0, lam, typ, use_ref=False):
    """TV energy (utils.c:60-117): type 1 = 2 lambda TV(u) + |u - u0|^2, type 2 = 2 lambda TV(u)."""
    lib, is_port = _lib(use_ref)
    u = np.ascontiguousarray(u, dtype=np.float32)
    u0 = np.ascontiguousarray(u0, dtype=np.float32)
    e = np.zeros(1, np.float32)
    if u.ndim == 2:
        fn = lib.port_TV_energy2D if is_port else lib.TV_energy2D
        fn(_ptr(u), _ptr(u0), _ptr(e), lam, typ, u.shape[1], u.shape[0])
    else:
        fn = lib.port_TV_energy3D if is_port else lib.TV_energy3D
        fn(_ptr(u), _ptr(u0), _ptr(e), lam, typ, u.shape[2], u.shape[1], u.shape[0])
    return float(e[0])


class WarmProx:
    """A regulariser whose state persists across calls, as in a prox session
    of the library: FGP keeps its last dual iterate P (the next call's R and
    P_prev start from it), SB its split and Bregman variables D, B, ROF and
    NDF (Jacobi order) start from the previous output.  The first call is
    the plain cold call.  `alg` is 0 ROF (lambda, tau), 1 FGP (lambda,
    methodTV, nonneg), 2 SB (mu, methodTV), 3 NDF (lambda, sigma, tau,
    penalty)."""

    def __init__(self, alg, params, shape):
        self.alg, self.prm = int(alg), [float(p) for p in params]
        self.shape = tuple(shape)
        n = int(np.prod(self.shape))
        na = 3 if len(self.shape) == 3 and self.shape[0] > 1 else 2
        self.state = np.zeros(n * (na if alg == 1 else 2 * na if alg == 2 else 0), np.float32)
        self.prev = None

    def __call__(self, z, iters):
        lib = port_lib()
        a, out, info = _prep(z)
        d = _dims(a)
        p = self.prm
        u0 = _ptr(self.prev) if self.prev is not None else None
        if self.alg == 0:
            lib.port_TV_ROF_init(_ptr(a), _ptr(out), _ptr(info), p[0], iters, p[1], 0.0, *d, u0)
        elif self.alg == 1:
            lib.port_TV_FGP_warm(_ptr(a), _ptr(out), _ptr(info), p[0], iters, 0.0, int(p[1]), int(p[2]), *d,
                                 _ptr(self.state))
        elif self.alg == 2:
            lib.port_SB_TV_warm(_ptr(a), _ptr(out), _ptr(info), p[0], iters, 0.0, int(p[1]), *d,
                                _ptr(self.state))
        else:
            lib.port_Diffusion_init(_ptr(a), _ptr(out), _ptr(info), p[0], p[1], iters, p[2], int(p[3]), 0.0, *d,
                                    u0)
        if self.alg in (0, 3):
            self.prev = out.copy()
        return out


def fista(alg, f, params, outer, inner, step):
    """FISTA on min_x 1/2 ||x - f||^2 + R(x) with warm-started proxes, in FP32
    as the library's session loop: z = y - step (y - f); x+ = prox(z) (inner
    iterations, warm state kept); t+ = (1 + sqrt(1 + 4 t^2)) / 2;
    y = x+ + ((t - 1) / t+)(x+ - x).  Starts from x = y = f, t = 1."""
    f = np.ascontiguousarray(f, dtype=np.float32)
    prox = WarmProx(alg, params, f.shape)
    x, y, t = f.copy(), f.copy(), np.float32(1.0)
    st = np.float32(step)
    for _ in range(outer):
        z = (y - st * (y - f)).astype(np.float32)
        xn = prox(z, inner)
        tn = np.float32((np.float32(1.0) + np.sqrt(np.float32(1.0) + np.float32(4.0) * t * t)) * np.float32(0.5))
        beta = np.float32((t - np.float32(1.0)) / tn)
        y = (xn + beta * (xn - x)).astype(np.float32)
        x, t = xn, tn
    return x


def admm(alg, f, params, outer, inner, rho, w=None):
    """ADMM (scaled form) on min_x 1/2 ||w^(1/2)(x - f)||^2 + rho R(x) with
    warm-started proxes of R, in FP32 as the library's session loop (each
    elementwise operation rounded separately): z = f, u = 0; per step
    x = (w f + rho (z - u)) / (w + rho), z = prox(x + u), u = (u + x) - z."""
    f = np.ascontiguousarray(f, dtype=np.float32)
    ww = np.ones_like(f) if w is None else np.ascontiguousarray(w, dtype=np.float32)
    prox = WarmProx(alg, params, f.shape)
    r = np.float32(rho)
    z, u = f.copy(), np.zeros_like(f)
    for _ in range(outer):
        x = ((ww * f) + (r * (z - u))) / (ww + r)
        v = x + u
        z = prox(v.astype(np.float32), inner)
        u = (u + x) - z
    return z


def pdhg(alg, f, params, outer, inner, tau, sigma, w=None):
    """PDHG (K = I) on min_x 1/2 ||w^(1/2)(x - f)||^2 + sigma R(x) with
    warm-started proxes of R, in FP32 as the library's session loop:
    x = xbar = f, y = 0; per step q = y * (1/sigma) + xbar,
    y = sigma (q - prox(q)), x+ = ((x - tau y) + (tau w) f) / (1 + tau w),
    xbar = 2 x+ - x."""
    f = np.ascontiguousarray(f, dtype=np.float32)
    ww = np.ones_like(f) if w is None else np.ascontiguousarray(w, dtype=np.float32)
    prox = WarmProx(alg, params, f.shape)
    t, sg = np.float32(tau), np.float32(sigma)
    inv_s = np.float32(1.0) / sg
    x, xbar, y = f.copy(), f.copy(), np.zeros_like(f)
    for _ in range(outer):
        q = (y * inv_s + xbar).astype(np.float32)
        p = prox(q, inner)
        y = sg * (q - p)
        tw = t * ww
        xn = ((x - t * y) + tw * f) / (np.float32(1.0) + tw)
        xbar = np.float32(2.0) * xn - x
        x = xn
    return x


def num_threads() -> int:
    return int(port_lib().port_num_threads())


class trace_checks:
    """Context manager recording every relative change the port's stopping
    rule evaluates: ``with trace_checks() as t: ...; t.values``."""

    def __init__(self, cap: int = 100000):
        self.buf = np.zeros(cap, dtype=np.float32)
        self.values = None

    def __enter__(self):
        port_lib().port_set_trace(_ptr(self.buf), self.buf.size)
        return self

    def __exit__(self, *exc):
        lib = port_lib()
        n = lib.port_trace_len()
        lib.port_set_trace(None, 0)
        self.values = self.buf[:n].copy()
        return False
