"""GPU tests of the next-tier entry points (LLT-ROF, FGP-dTV, TV energy)
beyond the golden cases of test_gpu_parity.py: odd shapes against the oracle
port, the host and device APIs against each other, and the energy against
the reference's own values."""
import ctypes

import numpy as np
import pytest

import cases as C
import oracle as O
from conftest import rel_tol

pytestmark = pytest.mark.gpu

SHAPES = [(40, 56), (1, 33), (33, 1), (10, 16, 22), (2, 30, 31), (3, 29, 15), (67, 70, 9), (130, 33, 35)]


LLT_SHAPES = SHAPES + [(67, 70, 10), (5, 31, 62), (3, 47, 2), (9, 1, 124), (4, 2, 90), (70, 29, 56)]


@pytest.mark.parametrize("shape", LLT_SHAPES, ids=str)
def test_llt_rof_matches_oracle_on_odd_shapes(shape):
    from ccpi.filters.regularisers import LLT_ROF

    rng = np.random.default_rng(41 + sum(shape))
    x = rng.random(shape).astype(np.float32)
    for epsil in (0.0, 1e-3):
        ref, iref = O.llt_rof(x, 0.02, 0.01, 80, 0.001, epsil)
        info = np.zeros(2, np.float32)
        got = LLT_ROF(x, 0.02, 0.01, 80, 0.001, epsil, device="gpu", infovector=info)
        assert int(info[0]) == int(iref[0])
        assert np.max(np.abs(got - ref)) <= rel_tol(ref, 1e-4)


@pytest.mark.parametrize("shape", LLT_SHAPES, ids=str)
def test_llt_rof_two_voxel_kernel_equals_one_voxel_kernel(shape, monkeypatch):
    """3D volumes with an even row length run the two-voxel LLT-ROF kernel by
    default; it computes the iteration of the one-voxel streaming kernel.  The
    LLT term dxx / (|dxx| + 1e-12) is the sign of dxx wherever |dxx| >> 1e-12,
    so a last-place rounding difference in a second difference near zero
    moves a voxel by up to 2 tau lambdaLLT per iteration: the bar is the
    oracle tests' 1e-4 of the range, not 1e-5."""
    from ccpi.filters.regularisers import LLT_ROF

    rng = np.random.default_rng(47 + sum(shape))
    x = rng.random(shape).astype(np.float32)
    for epsil in (0.0, 1e-3):
        ia, ib = np.zeros(2, np.float32), np.zeros(2, np.float32)
        a = LLT_ROF(x, 0.02, 0.01, 80, 0.001, epsil, device="gpu", infovector=ia)
        monkeypatch.setenv("CILREG_LLT_KERNEL", "stream")
        b = LLT_ROF(x, 0.02, 0.01, 80, 0.001, epsil, device="gpu", infovector=ib)
        monkeypatch.delenv("CILREG_LLT_KERNEL")
        assert int(ia[0]) == int(ib[0])
        assert np.max(np.abs(a - b)) <= rel_tol(b, 1e-4)


PAIR_2D_SHAPES = [(130, 98), (1, 64), (7, 2), (2, 90), (65, 300), (29, 58), (257, 510)]
PAIR_2D_CALLS = {
    "LLT_ROF": (lambda R, x, e, info: R.LLT_ROF(x, 0.02, 0.01, 60, 0.001, e, device="gpu", infovector=info),
                lambda x, e: O.llt_rof(x, 0.02, 0.01, 60, 0.001, e)),
    "Diff4th": (lambda R, x, e, info: R.Diff4th(x, 0.8, 0.02, 60, 1e-4, e, device="gpu", infovector=info),
                lambda x, e: O.diff4th(x, 0.8, 0.02, 60, 1e-4, e)),
    "FGP_iso_nonneg": (lambda R, x, e, info: R.FGP_TV(x, 0.05, 60, e, 0, 1, device="gpu", infovector=info),
                       lambda x, e: O.fgp_tv(x, 0.05, 60, e, 0, 1)),
    "FGP_aniso": (lambda R, x, e, info: R.FGP_TV(x, 0.05, 60, e, 1, 0, device="gpu", infovector=info),
                  lambda x, e: O.fgp_tv(x, 0.05, 60, e, 1, 0)),
    "FGP_dTV": (lambda R, x, e, info: R.FGP_dTV(x, np.ascontiguousarray(x[::-1, ::-1]), 0.05, 60, e, 0.2, 0, 1,
                                                device="gpu", infovector=info),
                lambda x, e: O.dtv_fgp(x, np.ascontiguousarray(x[::-1, ::-1]), 0.05, 60, e, 0.2, 0, 1)),
}


@pytest.mark.parametrize("shape", PAIR_2D_SHAPES, ids=str)
@pytest.mark.parametrize("reg", sorted(PAIR_2D_CALLS))
def test_two_pixel_2d_kernels_match_oracle(reg, shape):
    """2D images with an even row length run the two-pixel kernels
    (k_llt_pair2d, k_d4_pair2d, k_fgp_x2_2d, also for FGP-dTV): several tiles in x and y, rows of two
    pixels, a single row, against the oracle with the same stopping
    iteration."""
    from ccpi.filters import regularisers as R

    call, oracle = PAIR_2D_CALLS[reg]
    rng = np.random.default_rng(53 + sum(shape))
    x = rng.random(shape).astype(np.float32)
    for epsil in (0.0, 1e-3):
        ref, iref = oracle(x, epsil)
        info = np.zeros(2, np.float32)
        got = call(R, x, epsil, info)
        assert int(info[0]) == int(iref[0])
        assert np.max(np.abs(got - ref)) <= rel_tol(ref, 1e-4)


@pytest.mark.parametrize("reg", sorted(PAIR_2D_CALLS))
def test_two_pixel_2d_kernels_with_arrays_off_8_byte_alignment(reg):
    """An input 4 bytes off an 8-byte boundary runs the 4-byte variant of the
    2D two-pixel kernels, which gives the 8-byte variant's result bit for
    bit."""
    import torch
    from ccpi.filters import regularisersCuPy as D

    shape = (77, 130)
    n = shape[0] * shape[1]
    x = torch.from_numpy(np.random.default_rng(59).random(shape).astype(np.float32)).cuda()
    outs = []
    for off in (0, 1):
        buf = torch.zeros(n + 2, device="cuda")
        buf[off:off + n] = x.ravel()
        t = buf[off:off + n].view(shape)
        assert (t.data_ptr() % 8 == 0) == (off == 0)
        if reg == "LLT_ROF":
            outs.append(D.LLT_ROF(t, 0.02, 0.01, 40, 0.001))
        elif reg == "Diff4th":
            outs.append(D.Diff4th(t, 0.8, 0.02, 40, 1e-4))
        elif reg == "FGP_dTV":
            outs.append(D.FGP_dTV(t, t.flip(0).contiguous(), 0.05, 40, 0.0, 0.2, 0, 1))
        else:
            outs.append(D.FGP_TV(t, 0.05, 40, 0.0, 1 if "aniso" in reg else 0, 1 if "nonneg" in reg else 0))
    torch.cuda.synchronize()
    assert torch.equal(outs[0], outs[1])


@pytest.mark.parametrize("shape", SHAPES, ids=str)
def test_fgp_dtv_matches_oracle_on_odd_shapes(shape):
    from ccpi.filters.regularisers import FGP_dTV

    rng = np.random.default_rng(43 + sum(shape))
    x = rng.random(shape).astype(np.float32)
    r = rng.random(shape).astype(np.float32)
    for method, nonneg, epsil in ((0, 1, 3e-4), (1, 0, 0.0)):
        ref, iref = O.dtv_fgp(x, r, 0.05, 80, epsil, 0.2, method, nonneg)
        info = np.zeros(2, np.float32)
        got = FGP_dTV(x, r, 0.05, 80, epsil, 0.2, method, nonneg, device="gpu", infovector=info)
        assert int(info[0]) == int(iref[0])
        assert np.max(np.abs(got - ref)) <= rel_tol(ref, 1e-4)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("lam,typ", C.ENERGY)
def test_tv_energy_matches_reference(dim, lam, typ, golden):
    """The reference sums sequentially in FP32, the GPU in FP64: equal to 1e-5."""
    from ccpi.filters.regularisers import TV_ENERGY

    u, u0 = golden[f"input_{dim}d"], golden[f"ref_{dim}d"]
    e = float(TV_ENERGY(u, u0, lam, typ)[0])
    ref = float(golden[f"energy_{dim}d_{lam}_{typ}"])
    assert abs(e - ref) <= 1e-5 * abs(ref)
    exact = O.tv_energy(u.astype(np.float64).astype(np.float32), u0, lam, typ)  # port, same terms
    assert abs(e - exact) <= 1e-5 * abs(exact)


def test_tv_energy_large_volume_against_float64_sum():
    """At 2^24 voxels the FP64 accumulation stays at FP32 term rounding."""
    from ccpi.filters.regularisers import TV_ENERGY

    rng = np.random.default_rng(5)
    u = rng.random((256, 256, 256), dtype=np.float32)
    u0 = rng.random((256, 256, 256), dtype=np.float32)
    e = float(TV_ENERGY(u, u0, 0.1, 1)[0])
    ud = u.astype(np.float64)
    gx = np.diff(ud, axis=2, append=ud[:, :, -1:])
    gy = np.diff(ud, axis=1, append=ud[:, -1:, :])
    gz = np.diff(ud, axis=0, append=ud[-1:, :, :])
    exact = 2 * 0.1 * np.sqrt(gx * gx + gy * gy + gz * gz).sum() + ((ud - u0) ** 2).sum()
    assert abs(e - exact) <= 1e-6 * abs(exact)


def test_device_api_matches_host_api():
    import torch

    from ccpi.filters import utils as U
    from ccpi.filters.regularisers import FGP_dTV, LLT_ROF, TV_ENERGY

    rng = np.random.default_rng(9)
    x = rng.random((12, 40, 36)).astype(np.float32)
    r = rng.random((12, 40, 36)).astype(np.float32)
    dims = (36, 40, 12)
    s = torch.cuda.current_stream().cuda_stream
    dx, dr = torch.from_numpy(x).cuda(), torch.from_numpy(r).cuda()
    info = (ctypes.c_float * 2)()

    out = torch.zeros_like(dx)
    U.check_status(U.cilregcuda.cilreg_llt_rof_dev(dx.data_ptr(), out.data_ptr(), info, 0.02, 0.01, 50, 0.001, 0.0,
                                                   *dims, s))
    np.testing.assert_array_equal(out.cpu().numpy(), LLT_ROF(x, 0.02, 0.01, 50, 0.001, 0.0, device="gpu"))

    out = torch.zeros_like(dx)
    U.check_status(U.cilregcuda.cilreg_dtv_fgp_dev(dx.data_ptr(), dr.data_ptr(), out.data_ptr(), info, 0.05, 50,
                                                   0.0, 0.2, 0, 1, *dims, s))
    np.testing.assert_array_equal(out.cpu().numpy(), FGP_dTV(x, r, 0.05, 50, 0.0, 0.2, 0, 1, device="gpu"))

    e = (ctypes.c_float * 1)()
    U.check_status(U.cilregcuda.cilreg_tv_energy_dev(dx.data_ptr(), dr.data_ptr(), e, 0.1, 1, *dims, s))
    assert e[0] == TV_ENERGY(x, r, 0.1, 1)[0]


def test_cpu_abi_is_the_same_gpu_code():
    from ccpi.filters.regularisers import FGP_dTV, LLT_ROF

    rng = np.random.default_rng(10)
    x = rng.random((9, 30, 33)).astype(np.float32)
    r = rng.random((9, 30, 33)).astype(np.float32)
    np.testing.assert_array_equal(LLT_ROF(x, 0.02, 0.01, 40, 0.001, 1e-3, device="cpu"),
                                  LLT_ROF(x, 0.02, 0.01, 40, 0.001, 1e-3, device="gpu"))
    np.testing.assert_array_equal(FGP_dTV(x, r, 0.05, 40, 1e-4, 0.2, 0, 1, device="cpu"),
                                  FGP_dTV(x, r, 0.05, 40, 1e-4, 0.2, 0, 1, device="gpu"))


def test_invalid_arguments_raise():
    from ccpi.filters.regularisers import FGP_dTV, TV_ENERGY

    x = np.zeros((8, 9), np.float32)
    with pytest.raises(ValueError):
        FGP_dTV(x, np.zeros((9, 8), np.float32), 0.05, 10, 0.0, 0.2, 0, 0, device="gpu")
    with pytest.raises(ValueError):
        TV_ENERGY(x, x, 0.1, 3)


@pytest.mark.parametrize("shape", [(300, 300, 300), (97, 512, 515)], ids=str)
def test_large_host_arrays_match_the_device_call(shape):
    """Host-pointer calls on volumes of 100-500 MB (pageable arrays in, a
    fresh or caller-given output array out) return exactly the device-pointer
    call's result."""
    import torch
    from ccpi.filters import regularisersCuPy as D
    from ccpi.filters.regularisers import FGP_TV, ROF_TV

    rng = np.random.default_rng(sum(shape))
    x = rng.random(shape).astype(np.float32)
    ref = D.FGP_TV(torch.from_numpy(x).cuda(), 0.05, 6, 0.0, 0, 1).cpu().numpy()
    np.testing.assert_array_equal(FGP_TV(x, 0.05, 6, 0.0, 0, 1, device="gpu"), ref)
    out = np.empty_like(x)
    ROF_TV(x, 0.02, 5, 0.001, 0.0, device="gpu", out=out)
    np.testing.assert_array_equal(out, D.ROF_TV(torch.from_numpy(x).cuda(), 0.02, 5, 0.001).cpu().numpy())


def test_gpu_entry_points_start_u_prev_at_zero():
    """TV_FGP_GPU_main / dTV_FGP_GPU_main with a stopping rule take U_prev of
    iteration 0 as zero on the device (the reference GPU path leaves it
    uninitialised): whatever the caller's Output holds, the result and the
    stopping iteration are those of the C-OMP call with a zero Output."""
    from ccpi.filters.TV import TV_FGP_GPU, dTV_FGP_GPU
    from ccpi.filters.regularisers import FGP_TV, FGP_dTV

    rng = np.random.default_rng(5)
    x = rng.random((20, 24, 28)).astype(np.float32)
    r = rng.random((20, 24, 28)).astype(np.float32)
    ref_info = np.zeros(2, np.float32)
    ref = FGP_TV(x, 0.05, 60, 1e-3, 0, 1, device="cpu", infovector=ref_info)
    info = np.zeros(2, np.float32)
    got = TV_FGP_GPU(x, 0.05, 60, 1e-3, 0, 1, 0, out=rng.random(x.shape).astype(np.float32), infovector=info)
    np.testing.assert_array_equal(got, ref)
    assert int(info[0]) == int(ref_info[0])
    ref_info = np.zeros(2, np.float32)
    ref = FGP_dTV(x, r, 0.05, 60, 1e-3, 0.2, 0, 1, device="cpu", infovector=ref_info)
    got = dTV_FGP_GPU(x, r, 0.05, 60, 1e-3, 0.2, 0, 1, 0, out=rng.random(x.shape).astype(np.float32),
                      infovector=info)
    np.testing.assert_array_equal(got, ref)
    assert int(info[0]) == int(ref_info[0])
