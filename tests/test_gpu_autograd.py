"""The hand-written adjoint of unrolled FGP-TV (cilreg_fgp_tv_vjp_dev behind
torch.autograd.Function) against an FP64 unrolled oracle differentiated by
torch's own autograd, and against central finite differences (lambda step
1e-3 relative; directional step 1e-5, below the projections' kinks)."""
import numpy as np
import pytest

import fgp_torch64 as O64
from conftest import rel_tol

pytestmark = pytest.mark.gpu


def _relerr(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _problem(shape, seed):
    from ccpi.supp.phantoms import noisy_phantom

    f = noisy_phantom(shape, 6, seed)
    g = noisy_phantom(shape, 6, seed + 50)
    return f, g


def _gpu_grads(f, g, lam, iters, method, nonneg, ckpt):
    import torch
    from ccpi.filters.autograd import fgp_tv

    ft = torch.tensor(f, device="cuda", requires_grad=True)
    lt = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    y = fgp_tv(ft, lt, iters, method, nonneg, ckpt)
    loss = 0.5 * ((y.double() - torch.tensor(g, device="cuda", dtype=torch.float64)) ** 2).sum()
    loss.backward()
    return y.detach().cpu().numpy(), ft.grad.cpu().numpy(), float(lt.grad), float(loss.detach())


def _oracle_grads(f, g, lam, iters, method, nonneg):
    import torch

    f64 = torch.tensor(f, dtype=torch.float64, requires_grad=True)
    l64 = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    y = O64.fgp_unrolled(f64, l64, iters, method, nonneg)
    loss = 0.5 * ((y - torch.tensor(g, dtype=torch.float64)) ** 2).sum()
    loss.backward()
    return y.detach().numpy(), f64.grad.numpy(), float(l64.grad), float(loss)


CASES = [((10, 12, 14), 0, 0), ((10, 12, 14), 1, 1), ((9, 16, 13), 0, 1), ((24, 30), 0, 0), ((24, 30), 1, 1)]


@pytest.mark.parametrize("shape, method, nonneg", CASES, ids=[f"{s}-m{m}-n{n}" for s, m, n in CASES])
def test_adjoint_matches_fp64_oracle(shape, method, nonneg):
    f, g = _problem(shape, 21)
    iters, ckpt, lam = 30, 7, 0.05
    y, fb, lb, _ = _gpu_grads(f, g, lam, iters, method, nonneg, ckpt)
    y64, fb64, lb64, _ = _oracle_grads(f, g, lam, iters, method, nonneg)
    assert np.max(np.abs(y - y64)) <= rel_tol(y64, 1e-5)
    assert _relerr(fb, fb64) <= 1e-3
    assert abs(lb - lb64) <= 1e-3 * abs(lb64)


def test_oracle_forward_equals_c_port():
    import torch
    import oracle as O

    f, _ = _problem((10, 12, 14), 3)
    for method, nonneg in ((0, 0), (1, 1)):
        ref, _ = O.fgp_tv(f, 0.05, 25, 0.0, method, nonneg)
        y = O64.fgp_unrolled(torch.tensor(f, dtype=torch.float64), torch.tensor(0.05, dtype=torch.float64), 25,
                             method, nonneg).numpy()
        assert np.max(np.abs(y - ref)) <= rel_tol(ref, 1e-5)


def test_checkpoint_interval_does_not_change_gradients():
    f, g = _problem((10, 12, 14), 8)
    base = _gpu_grads(f, g, 0.04, 23, 0, 1, 23)
    for ckpt in (1, 4, 5):
        other = _gpu_grads(f, g, 0.04, 23, 0, 1, ckpt)
        np.testing.assert_array_equal(other[1], base[1])
        assert other[2] == base[2]


def test_central_differences_fp64_and_gpu():
    """dL/dlambda and a directional dL/df by central differences with steps of
    1e-3 relative to lambda and to the data scale.  The map is piecewise smooth
    (the projections have kinks), so larger absolute steps cross kinks."""
    import torch
    from ccpi.filters.autograd import fgp_tv

    f, g = _problem((8, 10, 12), 30)
    lam, iters = 0.05, 20
    h = 1e-3 * lam
    _, fb, lb, _ = _gpu_grads(f, g, lam, iters, 0, 0, 5)
    rng = np.random.default_rng(1)
    direction = rng.standard_normal(f.shape)

    def loss64(ff, ll):
        y = O64.fgp_unrolled(torch.tensor(ff, dtype=torch.float64), torch.tensor(ll, dtype=torch.float64), iters, 0, 0)
        return 0.5 * float(((y - torch.tensor(g, dtype=torch.float64)) ** 2).sum())

    fd_lam = (loss64(f, lam + h) - loss64(f, lam - h)) / (2 * h)
    hf = 1e-5  # a step along a random direction moves every voxel: keep it below the kinks
    fd_dir = (loss64(f + hf * direction, lam) - loss64(f - hf * direction, lam)) / (2 * hf)
    assert abs(lb - fd_lam) <= 1e-3 * abs(fd_lam)
    assert abs(float(np.sum(fb * direction)) - fd_dir) <= 1e-3 * abs(fd_dir)

    def loss_gpu(ll):
        with torch.no_grad():
            y = fgp_tv(torch.tensor(f, device="cuda"), ll, iters, 0, 0, 5)
        return 0.5 * float(((y.double().cpu().numpy() - g) ** 2).sum())

    fd_gpu = (loss_gpu(lam + h) - loss_gpu(lam - h)) / (2 * h)
    assert abs(lb - fd_gpu) <= 1e-2 * abs(fd_gpu)


def test_batched_volumes_and_learnable_lambda():
    """A batch (B, Z, Y, X) with one shared lambda: gradient = sum over volumes."""
    import torch
    from ccpi.filters.autograd import fgp_tv

    f1, g1 = _problem((8, 10, 12), 40)
    f2, g2 = _problem((8, 10, 12), 41)
    fb = torch.tensor(np.stack([f1, f2]), device="cuda", requires_grad=True)
    lt = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    y = fgp_tv(fb, lt, 15, 0, 1, 5, batched=True)
    target = torch.tensor(np.stack([g1, g2]), device="cuda", dtype=torch.float64)
    (0.5 * ((y.double() - target) ** 2).sum()).backward()
    s1 = _gpu_grads(f1, g1, 0.05, 15, 0, 1, 5)
    s2 = _gpu_grads(f2, g2, 0.05, 15, 0, 1, 5)
    np.testing.assert_array_equal(fb.grad[0].cpu().numpy(), s1[1])
    np.testing.assert_array_equal(fb.grad[1].cpu().numpy(), s2[1])
    assert abs(float(lt.grad) - (s1[2] + s2[2])) <= 1e-9 * abs(s1[2] + s2[2])


# ---------------------------------------------------------------------------
# ROF-TV adjoint (cilreg_rof_tv_vjp_dev behind ROFTVFunction)
#
# The ROF flux p / sqrt(p^2 + sum m^2 + 1e-8) turns into a step of width 1e-4
# where p is near zero and the minmods vanish, so on noisy data FP32 and FP64
# forward passes drift apart after a few dozen iterations and their
# linearisation points differ.  Two checks therefore: on smooth data
# (monotone along every axis, so the fluxes stay away from the step) the
# FP64 oracle's full gradient and central differences; on a noisy phantom,
# the FP64 oracle's per-step vector-Jacobian products chained along the
# GPU's own forward states.

import rof_torch64 as R64


def _smooth(shape, seed):
    rng = np.random.default_rng(seed)
    axes = np.meshgrid(*[np.linspace(0.0, 1.0, n) for n in shape], indexing="ij")
    slopes = rng.uniform(0.5, 1.0, len(shape))
    freqs = rng.uniform(2.0, 6.0, len(shape))
    f = sum(s * a for s, a in zip(slopes, axes))
    # curvature along every axis (no minmod ties), slope everywhere positive
    f = f + 0.04 * np.sin(sum(w * a for w, a in zip(freqs, axes)) + rng.uniform(0, 6.28))
    return f.astype(np.float32)


def _rof_gpu_grads(f, g, lam, iters, tau, ckpt):
    import torch
    from ccpi.filters.autograd import rof_tv

    ft = torch.tensor(f, device="cuda", requires_grad=True)
    lt = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    y = rof_tv(ft, lt, iters, tau, ckpt)
    loss = 0.5 * ((y.double() - torch.tensor(g, device="cuda", dtype=torch.float64)) ** 2).sum()
    loss.backward()
    return y.detach().cpu().numpy(), ft.grad.cpu().numpy(), float(lt.grad), float(loss.detach())


def _rof_oracle_grads(f, g, lam, iters, tau):
    import torch

    f64 = torch.tensor(f, dtype=torch.float64, requires_grad=True)
    l64 = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    y = R64.rof_unrolled(f64, l64, iters, tau)
    loss = 0.5 * ((y - torch.tensor(g, dtype=torch.float64)) ** 2).sum()
    loss.backward()
    return y.detach().numpy(), f64.grad.numpy(), float(l64.grad), float(loss)


ROF_SHAPES = [(10, 12, 14), (24, 30), (1, 9, 7), (9, 1, 13), (2, 6, 5)]


@pytest.mark.parametrize("shape", ROF_SHAPES, ids=str)
def test_rof_adjoint_matches_fp64_oracle_on_smooth_data(shape):
    f = _smooth(shape, 5)
    g = _smooth(shape, 6)[::-1].copy()
    iters, ckpt, lam, tau = 30, 7, 0.05, 0.01
    y, fb, lb, _ = _rof_gpu_grads(f, g, lam, iters, tau, ckpt)
    y64, fb64, lb64, _ = _rof_oracle_grads(f, g, lam, iters, tau)
    assert np.max(np.abs(y - y64)) <= rel_tol(y64, 1e-5)
    assert _relerr(fb, fb64) <= 1e-3
    assert abs(lb - lb64) <= 1e-3 * abs(lb64)


@pytest.mark.parametrize("shape", [(10, 12, 14), (24, 30)], ids=str)
def test_rof_adjoint_matches_chained_fp64_steps_on_noisy_data(shape):
    import torch
    from ccpi.filters.regularisersCuPy import ROF_TV

    f, g = _problem(shape, 23)
    iters, lam, tau = 20, 0.05, 0.01
    _, fb, lb, _ = _rof_gpu_grads(f, g, lam, iters, tau, 6)
    ft = torch.tensor(f, device="cuda")
    states = [f.astype(np.float64)] + [ROF_TV(ft, lam, k, tau).cpu().numpy().astype(np.float64)
                                       for k in range(1, iters + 1)]
    f64 = torch.tensor(f, dtype=torch.float64)
    w = torch.tensor(states[-1] - g.astype(np.float64))
    fbar = torch.zeros_like(f64)
    lbar = 0.0
    for k in range(iters - 1, -1, -1):
        uk = torch.tensor(states[k], requires_grad=True)
        fk = f64.clone().requires_grad_(True)
        lk = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
        step = R64.rof_step(uk, fk, lk, tau)
        gu, gf, gl = torch.autograd.grad(step, (uk, fk, lk), grad_outputs=w)
        fbar += gf
        lbar += float(gl)
        w = gu
    fbar += w
    assert _relerr(fb, fbar.numpy()) <= 1e-3
    assert abs(lb - lbar) <= 1e-3 * abs(lbar)


def test_rof_checkpoint_interval_does_not_change_gradients():
    f, g = _problem((10, 12, 14), 9)
    base = _rof_gpu_grads(f, g, 0.04, 23, 0.01, 23)
    for ckpt in (1, 4, 5, 40):
        other = _rof_gpu_grads(f, g, 0.04, 23, 0.01, ckpt)
        np.testing.assert_array_equal(other[1], base[1])
        assert other[2] == base[2]


def test_rof_central_differences_fp64_and_gpu():
    import torch
    from ccpi.filters.autograd import rof_tv

    f = _smooth((8, 10, 12), 31)
    g = _smooth((8, 10, 12), 32)[::-1].copy()
    lam, iters, tau = 0.05, 20, 0.01
    h = 1e-3 * lam
    _, fb, lb, _ = _rof_gpu_grads(f, g, lam, iters, tau, 5)
    # a direction that keeps every difference's sign and every minmod's
    # choice (a scaling of f plus ramps), so the step crosses no kink
    axes = np.meshgrid(*[np.linspace(0.0, 1.0, n) for n in f.shape], indexing="ij")
    direction = f.astype(np.float64) + 0.5 * axes[0] + 0.25 * axes[-1]

    def loss64(ff, ll):
        y = R64.rof_unrolled(torch.tensor(ff, dtype=torch.float64), torch.tensor(ll, dtype=torch.float64), iters, tau)
        return 0.5 * float(((y - torch.tensor(g, dtype=torch.float64)) ** 2).sum())

    fd_lam = (loss64(f, lam + h) - loss64(f, lam - h)) / (2 * h)
    hf = 1e-5
    fd_dir = (loss64(f + hf * direction, lam) - loss64(f - hf * direction, lam)) / (2 * hf)
    assert abs(lb - fd_lam) <= 1e-3 * abs(fd_lam)
    assert abs(float(np.sum(fb * direction)) - fd_dir) <= 1e-3 * abs(fd_dir)

    def loss_gpu(ll):
        with torch.no_grad():
            y = rof_tv(torch.tensor(f, device="cuda"), ll, iters, tau, 5)
        return 0.5 * float(((y.double().cpu().numpy() - g) ** 2).sum())

    hg = 1e-2 * lam  # FP32 forward: a larger step
    fd_gpu = (loss_gpu(lam + hg) - loss_gpu(lam - hg)) / (2 * hg)
    assert abs(lb - fd_gpu) <= 1e-2 * abs(fd_gpu)


def test_rof_batched_volumes_and_learnable_lambda():
    import torch
    from ccpi.filters.autograd import rof_tv

    f1, g1 = _problem((8, 10, 12), 42)
    f2, g2 = _problem((8, 10, 12), 43)
    fb = torch.tensor(np.stack([f1, f2]), device="cuda", requires_grad=True)
    lt = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    y = rof_tv(fb, lt, 15, 0.01, 5, batched=True)
    target = torch.tensor(np.stack([g1, g2]), device="cuda", dtype=torch.float64)
    (0.5 * ((y.double() - target) ** 2).sum()).backward()
    s1 = _rof_gpu_grads(f1, g1, 0.05, 15, 0.01, 5)
    s2 = _rof_gpu_grads(f2, g2, 0.05, 15, 0.01, 5)
    np.testing.assert_array_equal(fb.grad[0].cpu().numpy(), s1[1])
    np.testing.assert_array_equal(fb.grad[1].cpu().numpy(), s2[1])
    assert abs(float(lt.grad) - (s1[2] + s2[2])) <= 1e-9 * abs(s1[2] + s2[2])


def test_rof_vjp_rejects_bad_arguments():
    import ctypes

    import torch
    from ccpi.filters.utils import cilregcuda

    x = torch.zeros((4, 5, 6), device="cuda")
    lb = ctypes.c_double(0.0)
    s = torch.cuda.current_stream().cuda_stream
    fn = cilregcuda.cilreg_rof_tv_vjp_dev
    assert fn(x.data_ptr(), x.data_ptr(), x.data_ptr(), ctypes.byref(lb), 0.05, 0, 0.01, 5, 6, 5, 4, s) == -2
    assert fn(x.data_ptr(), x.data_ptr(), x.data_ptr(), ctypes.byref(lb), 0.05, 10, 0.01, 0, 6, 5, 4, s) == -2
    assert fn(None, x.data_ptr(), x.data_ptr(), ctypes.byref(lb), 0.05, 10, 0.01, 5, 6, 5, 4, s) == -2
