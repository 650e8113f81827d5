"""Parity case table shared by the fixture generator and the tests.

Every case is one call of a regulariser with the reference's argument
meanings.  Inputs are seeded ellipse/ellipsoid phantoms with Gaussian noise
(sigma 0.05); the iteration counts and tolerances are chosen so that each
stopping case fires well before its cap.  Parameter values for the fixed-count
cases follow the reference's own tests (test/test_2d_cpu_vs_gpu.py:56-505,
test/test_3d_cpu_vs_gpu.py:61-125), with fewer iterations.
"""
from __future__ import annotations

SHAPE_2D = (40, 56)       # (Y, X)
SHAPE_3D = (10, 16, 22)   # (Z, Y, X)
SEEDS = {2: (6, 11), 3: (8, 12)}  # (number of shapes, seed)
# a second 3D input whose x extent is a multiple of 4, the volumes the kernels
# that stage their inputs by tensor copies run on (FGP, TGV)
SHAPE_3D_X4 = (10, 16, 24)
SEED_3D_X4 = (8, 13)
STAGED = ("fgp_iso", "fgp_aniso_nonneg", "fgp_stop", "tgv", "tgv_stop")


def _c(name, alg, **p):
    return {"name": name, "alg": alg, "params": p}


_BASE = [
    _c("rof", "rof", lam=0.02, iters=200, tau=0.001, epsil=0.0),
    _c("rof_stop", "rof", lam=0.02, iters=300, tau=0.001, epsil=1e-3),
    _c("fgp_iso", "fgp", lam=0.05, iters=120, epsil=0.0, method=0, nonneg=0),
    _c("fgp_aniso_nonneg", "fgp", lam=0.05, iters=120, epsil=0.0, method=1, nonneg=1),
    _c("fgp_stop", "fgp", lam=0.05, iters=300, epsil=3e-4, method=0, nonneg=1),
    _c("pd_iso", "pd", lam=0.05, iters=120, epsil=0.0, lipschitz=8.0, method=0, nonneg=0),
    _c("pd_aniso_nonneg", "pd", lam=0.05, iters=120, epsil=0.0, lipschitz=8.0, method=1, nonneg=1),
    _c("pd_stop", "pd", lam=0.05, iters=300, epsil=3e-4, lipschitz=8.0, method=0, nonneg=1),
    _c("sb_iso", "sb", mu=0.05, iters=60, epsil=0.0, method=0),
    _c("sb_aniso", "sb", mu=0.05, iters=60, epsil=0.0, method=1),
    _c("sb_stop", "sb", mu=0.05, iters=300, epsil=3e-4, method=0),
    _c("tgv", "tgv", lam=0.05, alpha1=1.0, alpha0=2.0, iters=120, L2=12.0, epsil=0.0),
    _c("tgv_stop", "tgv", lam=0.05, alpha1=1.0, alpha0=2.0, iters=300, L2=12.0, epsil=3e-3),
    _c("ndf_linear", "ndf", lam=0.02, sigma=0.0, iters=100, tau=0.01, penalty=1, epsil=0.0),
    _c("ndf_huber", "ndf", lam=0.02, sigma=0.05, iters=100, tau=0.01, penalty=1, epsil=0.0),
    _c("ndf_pm", "ndf", lam=0.02, sigma=0.05, iters=100, tau=0.01, penalty=2, epsil=0.0),
    _c("ndf_tukey", "ndf", lam=0.02, sigma=0.05, iters=100, tau=0.01, penalty=3, epsil=0.0),
    _c("ndf_thrlin", "ndf", lam=0.02, sigma=0.05, iters=100, tau=0.01, penalty=4, epsil=0.0),
    _c("ndf_thrhuber", "ndf", lam=0.02, sigma=0.05, iters=100, tau=0.01, penalty=5, epsil=0.0),
    _c("ndf_stop", "ndf", lam=0.02, sigma=0.05, iters=300, tau=0.01, penalty=1, epsil=1e-3),
    _c("d4", "d4", lam=0.8, sigma=0.02, iters=120, tau=1e-4, epsil=0.0),
    _c("d4_stop", "d4", lam=0.8, sigma=0.02, iters=300, tau=1e-4, epsil=1e-3),
    # next-tier regularisers (reference test/test_2d_cpu_vs_gpu.py:361-377, 549-565)
    _c("llt_rof", "llt", lam_rof=0.02, lam_llt=0.01, iters=200, tau=0.001, epsil=0.0),
    _c("llt_rof_stop", "llt", lam_rof=0.02, lam_llt=0.01, iters=300, tau=0.001, epsil=1e-3),
    _c("dtv_iso", "dtv", lam=0.05, iters=120, epsil=0.0, eta=0.2, method=0, nonneg=0),
    _c("dtv_aniso_nonneg", "dtv", lam=0.05, iters=120, epsil=0.0, eta=0.2, method=1, nonneg=1),
    _c("dtv_stop", "dtv", lam=0.05, iters=300, epsil=3e-4, eta=0.2, method=0, nonneg=1),
]

# TV energy cases (lambda, type) on (input, reference image)
ENERGY = [(0.1, 1), (0.1, 2), (0.03, 1)]


def cases():
    out = []
    for dim in (2, 3):
        for c in _BASE:
            d = dict(c)
            d["dim"] = dim
            d["key"] = f"{c['name']}_{dim}d"
            out.append(d)
    return out


def staged_cases():
    """The FGP and TGV cases on the 3D input of x extent 24 (key suffix 3dx4)."""
    out = []
    for c in _BASE:
        if c["name"] in STAGED:
            d = dict(c)
            d["dim"] = 3
            d["key"] = f"{c['name']}_3dx4"
            out.append(d)
    return out


def make_input(dim: int):
    from ccpi.supp.phantoms import noisy_phantom

    n, seed = SEEDS[dim]
    return noisy_phantom(SHAPE_2D if dim == 2 else SHAPE_3D, n, seed)


def make_input_x4():
    from ccpi.supp.phantoms import noisy_phantom

    n, seed = SEED_3D_X4
    return noisy_phantom(SHAPE_3D_X4, n, seed)


def make_ref(dim: int, shape=None):
    """The FGP-dTV reference image: the noise-free phantom behind make_input
    (of `shape` instead of the case shape when given)."""
    from ccpi.supp.phantoms import clean_phantom

    n, seed = SEEDS[dim]
    return clean_phantom(shape or (SHAPE_2D if dim == 2 else SHAPE_3D), n, seed)


def _ref_for(case, x, ref):
    return make_ref(case["dim"], tuple(x.shape)) if ref is None else ref


def run_oracle(case, x, use_ref=False, jacobi=True, ref=None):
    """Run `case` on the oracle (port, or the compiled reference)."""
    import oracle as O

    p = case["params"]
    a = case["alg"]
    if a == "llt":
        return O.llt_rof(x, p["lam_rof"], p["lam_llt"], p["iters"], p["tau"], p["epsil"], use_ref=use_ref)
    if a == "dtv":
        r = _ref_for(case, x, ref)
        return O.dtv_fgp(x, r, p["lam"], p["iters"], p["epsil"], p["eta"], p["method"], p["nonneg"],
                         use_ref=use_ref)
    if a == "rof":
        return O.rof_tv(x, p["lam"], p["iters"], p["tau"], p["epsil"], use_ref=use_ref)
    if a == "fgp":
        return O.fgp_tv(x, p["lam"], p["iters"], p["epsil"], p["method"], p["nonneg"], use_ref=use_ref)
    if a == "pd":
        return O.pd_tv(x, p["lam"], p["iters"], p["epsil"], p["lipschitz"], p["method"], p["nonneg"], use_ref=use_ref)
    if a == "sb":
        return O.sb_tv(x, p["mu"], p["iters"], p["epsil"], p["method"], use_ref=use_ref)
    if a == "tgv":
        return O.tgv(x, p["lam"], p["alpha1"], p["alpha0"], p["iters"], p["L2"], p["epsil"], use_ref=use_ref)
    if a == "ndf":
        return O.ndf(x, p["lam"], p["sigma"], p["iters"], p["tau"], p["penalty"], p["epsil"], jacobi=jacobi,
                     use_ref=use_ref)
    if a == "d4":
        return O.diff4th(x, p["lam"], p["sigma"], p["iters"], p["tau"], p["epsil"], use_ref=use_ref)
    raise KeyError(a)


def run_gpu(case, x, api="gpu", device=0, ref=None):
    """Run `case` through the product's Python API.  api: 'gpu' (the *_GPU_main
    argument list), 'cpu' (the *_CPU_main list, which also runs on the GPU)."""
    import numpy as np
    from ccpi.filters import regularisers as R

    p = case["params"]
    a = case["alg"]
    info = np.zeros(2, np.float32)
    dev = "cpu" if api == "cpu" else device
    if a == "rof":
        out = R.ROF_TV(x, p["lam"], p["iters"], p["tau"], p["epsil"], device=dev, infovector=info)
    elif a == "fgp":
        out = R.FGP_TV(x, p["lam"], p["iters"], p["epsil"], p["method"], p["nonneg"], device=dev, infovector=info)
    elif a == "pd":
        if api == "cpu":
            out = R.PD_TV(x, p["lam"], p["iters"], p["epsil"], p["lipschitz"], p["method"], p["nonneg"], device=dev,
                          infovector=info)
        else:
            out = R.PD_TV(x, p["lam"], p["iters"], p["epsil"], p["lipschitz"], p["method"], p["nonneg"], device=dev,
                          infovector=info)
    elif a == "sb":
        out = R.SB_TV(x, p["mu"], p["iters"], p["epsil"], p["method"], device=dev, infovector=info)
    elif a == "tgv":
        out = R.TGV(x, p["lam"], p["alpha1"], p["alpha0"], p["iters"], p["L2"], p["epsil"], device=dev,
                    infovector=info)
    elif a == "ndf":
        out = R.NDF(x, p["lam"], p["sigma"], p["iters"], p["tau"], p["penalty"], p["epsil"], device=dev,
                    infovector=info)
    elif a == "d4":
        out = R.Diff4th(x, p["lam"], p["sigma"], p["iters"], p["tau"], p["epsil"], device=dev, infovector=info)
    elif a == "llt":
        out = R.LLT_ROF(x, p["lam_rof"], p["lam_llt"], p["iters"], p["tau"], p["epsil"], device=dev,
                        infovector=info)
    elif a == "dtv":
        r = _ref_for(case, x, ref)
        out = R.FGP_dTV(x, r, p["lam"], p["iters"], p["epsil"], p["eta"], p["method"], p["nonneg"], device=dev,
                        infovector=info)
    else:
        raise KeyError(a)
    return out, info
