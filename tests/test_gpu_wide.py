"""Volumes of 2^31 voxels or more: the paths with 64-bit element offsets.

A full-size oracle run is out of reach at this size, so each case uses a
size-independent property instead.  After k iterations a voxel depends only
on input voxels a few planes away (at most 4 planes per iteration for the
regularisers here), so a run on a window of the volume's planes reproduces
the full run on the window's planes that lie more than 4k planes from a cut
the window makes.  Each case runs the full volume once and compares three
80-plane windows (bottom, middle and top; the top one spans element offset 2^31)
with runs on the window alone.  The window runs are small (32-bit offsets)
and use the kernels the full run uses at this size: the register-pipelined
ROF kernel and the per-voxel SB, TGV and NDF kernels, which the full volume
selects, are forced for the windows through the kernel-selection variables.
Both runs use a stopping tolerance that is never met, so the stopping-check
variants (64-bit) run too.  Tolerance: 1e-6 of the data range (the same
arithmetic per voxel; an index error shows as an O(1) difference).
"""
import os

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SHAPE3 = (2049, 1024, 1024)  # 2,148,532,224 voxels; plane 2048 starts at offset 2^31
SHAPE2 = (32769, 65536)  # 2,147,549,184 pixels; row 32768 starts at offset 2^31
ITERS = 6  # stopping checks at iterations 0 and 5
EPSIL = 1e-20  # never met: the check kernels run, the runs do not stop
WIN, KEEP = 80, 16  # planes of a window; planes compared in it
REACH = 4  # planes a voxel's value reaches per iteration (at most)


def _cases():
    from ccpi.filters import regularisersCuPy as R

    # name: (call(x, ref, info), kernel variable and value that the full-size run implies)
    return {
        "ROF_TV": (lambda x, r, i: R.ROF_TV(x, 0.02, ITERS, 0.001, tolerance_param=EPSIL, infovector=i),
                   ("CILREG_ROF_KERNEL", "reg")),
        "FGP_TV": (lambda x, r, i: R.FGP_TV(x, 0.03, ITERS, EPSIL, 0, 1, infovector=i), None),
        "PD_TV": (lambda x, r, i: R.PD_TV(x, 0.03, ITERS, EPSIL, 0, 1, 8.0, infovector=i), None),
        "SB_TV": (lambda x, r, i: R.SB_TV(x, 0.03, ITERS, EPSIL, 0, infovector=i), ("CILREG_SB_KERNEL", "simple")),
        "TGV": (lambda x, r, i: R.TGV(x, 0.03, 1.0, 2.0, ITERS, 12.0, EPSIL, infovector=i),
                ("CILREG_TGV_KERNEL", "simple")),
        "NDF": (lambda x, r, i: R.NDF(x, 0.02, 0.02, ITERS, 0.01, 1, EPSIL, infovector=i),
                ("CILREG_NDF_KERNEL", "simple")),
        "Diff4th": (lambda x, r, i: R.Diff4th(x, 0.8, 0.02, ITERS, 0.0001, EPSIL, infovector=i), None),
        "LLT_ROF": (lambda x, r, i: R.LLT_ROF(x, 0.02, 0.01, ITERS, 0.001, EPSIL, infovector=i), None),
        "FGP_dTV": (lambda x, r, i: R.FGP_dTV(x, r, 0.05, ITERS, EPSIL, 0.2, 0, 1, infovector=i), None),
    }


NAMES = ["ROF_TV", "FGP_TV", "PD_TV", "SB_TV", "TGV", "NDF", "Diff4th", "LLT_ROF", "FGP_dTV"]


def _free():
    from ccpi.filters.utils import release_cached

    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    release_cached(0)


@pytest.fixture(scope="module", params=[3, 2], ids=["3d", "2d"])
def wide_input(request):
    import numpy as np

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    free, _ = torch.cuda.mem_get_info()
    if free < 200 * 2**30:
        pytest.skip(f"needs about 200 GB free on the device, {free / 2**30:.0f} GiB free")
    shape = SHAPE3 if request.param == 3 else SHAPE2
    g = torch.Generator(device="cuda").manual_seed(7 + request.param)
    x = torch.rand(shape, generator=g, device="cuda", dtype=torch.float32)
    r = torch.rand(shape, generator=g, device="cuda", dtype=torch.float32)
    assert x.numel() >= 2**31
    yield x, r, np
    del x, r
    _free()


@pytest.mark.parametrize("name", NAMES)
def test_wide_volume_matches_windows(name, wide_input):
    x, r, np = wide_input
    call, env = _cases()[name]
    info = np.zeros(2, np.float32)
    full = call(x, r, info)
    torch.cuda.synchronize()
    assert int(info[0]) == ITERS, info
    n0 = x.shape[0]
    margin = REACH * ITERS + 1
    # (first plane of the window, planes compared) for bottom, middle, top
    windows = [(0, (0, KEEP)),
               (n0 // 2 - WIN // 2, (n0 // 2 - KEEP // 2, n0 // 2 + KEEP // 2)),
               (n0 - WIN, (n0 - KEEP, n0))]
    old = os.environ.get(env[0]) if env else None
    try:
        if env:
            os.environ[env[0]] = env[1]
        for w0, (c0, c1) in windows:
            # the compared planes are at least `margin` planes from every cut
            # the window makes (a cut at 0 or n0 is the volume's own edge)
            assert (w0 == 0 or c0 - w0 >= margin) and (w0 + WIN == n0 or w0 + WIN - c1 >= margin)
            xs = x[w0:w0 + WIN].contiguous()
            rs = r[w0:w0 + WIN].contiguous()
            winfo = np.zeros(2, np.float32)
            part = call(xs, rs, winfo)
            a = full[c0:c1]
            b = part[c0 - w0:c1 - w0]
            rng = float(b.max() - b.min())
            diff = float((a - b).abs().max())
            assert int(winfo[0]) == ITERS
            assert diff <= 1e-6 * max(rng, 1e-12), (name, w0, diff, rng)
    finally:
        if env:
            if old is None:
                os.environ.pop(env[0], None)
            else:
                os.environ[env[0]] = old
    del full
    _free()
