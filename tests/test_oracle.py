"""CPU tests of the oracle: the C restatement must reproduce the reference's
own C-OMP outputs (golden fixtures made by tests/golden/make_golden.py from
the reference sources), before it is trusted as the GPU checker."""
import platform

import numpy as np
import pytest

import cases as C
import oracle as O
from conftest import rel_tol


def _bit_exact_platform():
    # the fixtures were made on x86-64; the port reproduces them bit for bit there
    return platform.machine() in ("x86_64", "AMD64")


@pytest.mark.parametrize("case", C.cases(), ids=lambda c: c["key"])
def test_port_matches_reference_fixture(case, golden):
    x = golden[f"input_{case['dim']}d"]
    out, info = C.run_oracle(case, x, use_ref=False, jacobi=False)
    ref = golden[f"out_{case['key']}"]
    ref_info = golden[f"info_{case['key']}"]
    assert out.shape == ref.shape
    assert int(info[0]) == int(ref_info[0])
    if _bit_exact_platform():
        np.testing.assert_array_equal(out, ref)
        assert info[1] == ref_info[1]
    else:
        assert np.max(np.abs(out - ref)) <= rel_tol(ref, 1e-6)


def test_fixture_inputs_are_the_seeded_phantoms(golden):
    for dim in (2, 3):
        np.testing.assert_array_equal(C.make_input(dim), golden[f"input_{dim}d"])
    np.testing.assert_array_equal(C.make_input_x4(), golden["input_3dx4"])


@pytest.mark.parametrize("case", C.staged_cases(), ids=lambda c: c["key"])
def test_port_matches_reference_fixture_x4(case, golden):
    """The FGP and TGV cases on the 3D input whose x extent is a multiple of 4."""
    x = golden["input_3dx4"]
    out, info = C.run_oracle(case, x, use_ref=False, jacobi=False)
    ref = golden[f"out_{case['key']}"]
    ref_info = golden[f"info_{case['key']}"]
    assert int(info[0]) == int(ref_info[0])
    if _bit_exact_platform():
        np.testing.assert_array_equal(out, ref)
    else:
        assert np.max(np.abs(out - ref)) <= rel_tol(ref, 1e-6)


ODD_SHAPES = [(3, 5), (7, 2), (2, 3, 5), (5, 4, 3), (13, 9, 2)]


@pytest.mark.parametrize("shape", ODD_SHAPES)
def test_port_matches_live_reference_on_odd_shapes(shape):
    """Against the reference compiled here (skipped where its sources are absent)."""
    if O.ref_lib() is None:
        pytest.skip("reference C-OMP library not built on this machine")
    rng = np.random.default_rng(sum(shape))
    x = rng.random(shape).astype(np.float32)
    checks = [
        (O.rof_tv, (0.02, 30, 0.001, 1e-4)),
        (O.fgp_tv, (0.05, 30, 1e-4, 0, 1)),
        (O.pd_tv, (0.05, 30, 1e-4, 8.0, 1, 0)),
        (O.sb_tv, (0.05, 20, 1e-4, 0)),
        (O.tgv, (0.05, 1.0, 2.0, 30, 12.0, 1e-4)),
        (O.diff4th, (0.8, 0.02, 30, 1e-4, 1e-4)),
    ]
    for fn, args in checks:
        a, ia = fn(x, *args)
        b, ib = fn(x, *args, use_ref=True)
        np.testing.assert_array_equal(a, b, err_msg=fn.__name__)
        np.testing.assert_array_equal(ia, ib, err_msg=fn.__name__)


def test_ndf_jacobi_close_to_lexicographic():
    """The Jacobi order (GPU semantics) and the reference's in-place order differ
    by O(tau) per sweep; on the fixture they stay within 1e-3 of the range."""
    x = C.make_input(2)
    for pen in (1, 2, 3, 4, 5):
        a, _ = O.ndf(x, 0.02, 0.05, 100, 0.01, pen, 0.0, jacobi=True)
        b, _ = O.ndf(x, 0.02, 0.05, 100, 0.01, pen, 0.0, jacobi=False)
        assert np.max(np.abs(a - b)) <= rel_tol(b, 1e-3)


def test_trace_records_every_check():
    x = C.make_input(2)
    with O.trace_checks() as t:
        _, info = O.fgp_tv(x, 0.05, 300, 3e-4, 0, 1)
    n_checks = int(info[0]) // 5 + 1
    assert t.values.size == n_checks
    assert t.values[-1] == info[1]
    assert np.sum(t.values < 3e-4) == 4  # the rule stops on the fourth hit


def test_zero_iterations_copies_input():
    x = C.make_input(3)
    out, info = O.rof_tv(x, 0.02, 0, 0.001, 0.0)
    np.testing.assert_array_equal(out, x)
    assert info[0] == 0


def test_invalid_penalty_rejected_by_port():
    x = C.make_input(2)
    lib = O.port_lib()
    a, out, info = O._prep(x)
    r = lib.port_Diffusion(O._ptr(a), O._ptr(out), O._ptr(info), 0.02, 0.05, 10, 0.01, 9, 0.0, *O._dims(a), 1)
    assert r < 0


@pytest.mark.parametrize("shape", [(40, 56), (3, 5), (10, 16, 22), (5, 4, 3), (13, 9, 2)])
def test_port_matches_live_reference_llt_dtv_energy(shape):
    """LLT-ROF, FGP-dTV and the TV energy of the port against the reference
    compiled here (skipped where its sources are absent).  Axes of length 1
    are left out: there the reference indexes outside the array."""
    if O.ref_lib() is None:
        pytest.skip("reference C-OMP library not built on this machine")
    rng = np.random.default_rng(7 + sum(shape))
    x = rng.random(shape).astype(np.float32)
    ref = rng.random(shape).astype(np.float32)
    for epsil in (0.0, 1e-3):
        a, ia = O.llt_rof(x, 0.02, 0.01, 40, 0.002, epsil)
        b, ib = O.llt_rof(x, 0.02, 0.01, 40, 0.002, epsil, use_ref=True)
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(ia, ib)
        for method, nonneg in ((0, 1), (1, 0)):
            a, ia = O.dtv_fgp(x, ref, 0.05, 40, epsil, 0.2, method, nonneg)
            b, ib = O.dtv_fgp(x, ref, 0.05, 40, epsil, 0.2, method, nonneg, use_ref=True)
            np.testing.assert_array_equal(a, b)
            np.testing.assert_array_equal(ia, ib)
    for typ in (1, 2):
        assert O.tv_energy(x, ref, 0.1, typ) == O.tv_energy(x, ref, 0.1, typ, use_ref=True)


def test_fixture_reference_images_are_the_clean_phantoms(golden):
    for dim in (2, 3):
        np.testing.assert_array_equal(C.make_ref(dim), golden[f"ref_{dim}d"])


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("lam,typ", C.ENERGY)
def test_port_energy_matches_reference_fixture(dim, lam, typ, golden):
    e = O.tv_energy(golden[f"input_{dim}d"], golden[f"ref_{dim}d"], lam, typ)
    ref = float(golden[f"energy_{dim}d_{lam}_{typ}"])
    if _bit_exact_platform():
        assert np.float32(e) == np.float32(ref)
    else:
        assert abs(e - ref) <= 1e-5 * abs(ref)


@pytest.mark.parametrize("shape", [(10, 12, 14), (24, 30), (1, 9, 7), (9, 1, 13), (2, 6, 5)], ids=str)
def test_rof_fp64_unrolled_oracle_matches_port(shape):
    """The FP64 torch restatement used to check the ROF adjoint computes the
    port's map: within 1e-5 of the range on a noisy phantom over 5 iterations
    (after a few dozen, FP32 and FP64 drift apart where the flux turns into a
    step) and on smooth data over 30."""
    torch = pytest.importorskip("torch")
    import rof_torch64 as R64
    from ccpi.supp.phantoms import noisy_phantom

    rng = np.random.default_rng(sum(shape))
    noisy = noisy_phantom(shape, 6, 3) if min(shape) > 1 else rng.random(shape).astype(np.float32)
    axes = np.meshgrid(*[np.linspace(0.0, 1.0, n) for n in shape], indexing="ij")
    smooth = (sum((0.5 + 0.1 * i) * a for i, a in enumerate(axes))
              + 0.04 * np.sin(sum((2.0 + i) * a for i, a in enumerate(axes)))).astype(np.float32)
    for f, iters in ((noisy, 5), (smooth, 30)):
        ref, _ = O.rof_tv(f, 0.05, iters, 0.01, 0.0)
        y = R64.rof_unrolled(torch.tensor(f, dtype=torch.float64), torch.tensor(0.05, dtype=torch.float64), iters,
                             0.01).numpy()
        assert np.max(np.abs(y - ref)) <= rel_tol(ref, 1e-5)


def test_llt_term_is_a_sign_copy_from_two_to_the_minus_15():
    """The two-voxel LLT-ROF kernel takes v / (|v| + 1e-12) as +-1 for
    |v| >= 2^-15 and as v for v = +-0, dividing only otherwise: in FP32 the
    IEEE quotient has exactly those values, and just below 2^-15 it does not."""
    rng = np.random.default_rng(13)
    e = rng.uniform(-15, 127, 3_000_000)
    v = (np.where(rng.random(e.size) < 0.5, -1.0, 1.0) * 2.0 ** e).astype(np.float32)
    v = v[np.isfinite(v) & (np.abs(v) >= np.float32(2.0 ** -15))]
    eps = np.float32(1e-12)
    with np.errstate(over="ignore"):
        np.testing.assert_array_equal(v / (np.abs(v) + eps), np.sign(v))
    z = np.float32([0.0, -0.0])
    q = z / (np.abs(z) + eps)
    np.testing.assert_array_equal(np.signbit(q), np.signbit(z))
    below = np.nextafter(np.float32(2.0 ** -15), np.float32(0))
    assert below / (below + eps) != np.float32(1.0)


def test_anisotropic_projection_is_a_clip_without_division():
    """The kernels take p / max(|p|, 1) as p for |p| <= 1 and as +-1 beyond:
    in FP32 the IEEE quotient has exactly those values."""
    rng = np.random.default_rng(14)
    e = rng.uniform(-40, 127, 3_000_000)
    p = (np.where(rng.random(e.size) < 0.5, -1.0, 1.0) * 2.0 ** e).astype(np.float32)
    p = np.concatenate([p[np.isfinite(p)], np.float32([0.0, -0.0, 1.0, -1.0]),
                        np.nextafter(np.float32([1.0, -1.0]), np.float32(0)),
                        np.nextafter(np.float32([1.0, -1.0]), np.float32([2.0, -2.0]))])
    q = p / np.maximum(np.abs(p), np.float32(1.0))
    clip = np.where(np.abs(p) <= 1, p, np.sign(p)).astype(np.float32)
    np.testing.assert_array_equal(q, clip)
    np.testing.assert_array_equal(np.signbit(q), np.signbit(clip))
