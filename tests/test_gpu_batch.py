"""GPU tests of the batched API: many volumes of uneven shape in one call give
the single-volume results (same kernels, per-volume stopping rules), with and
without the CUDA graph and the z-chunk autotuner."""
import numpy as np
import pytest

from conftest import rel_tol

pytestmark = pytest.mark.gpu


def _volumes(shapes, seed):
    rng = np.random.default_rng(seed)
    return [rng.random(s).astype(np.float32) for s in shapes]


SHAPES_3D = [(17, 30, 41), (64, 33, 20), (9, 9, 70), (40, 40, 40), (3, 200, 31)]
SHAPES_2D = [(37, 51), (128, 9), (200, 200), (1, 77)]


@pytest.mark.parametrize("shapes", [SHAPES_3D, SHAPES_2D], ids=["3d", "2d"])
@pytest.mark.parametrize("epsil", [0.0, 3e-4])
def test_fgp_batch_equals_single_calls(shapes, epsil, monkeypatch):
    from ccpi.filters.batch import FGP_TV_batch
    from ccpi.filters.regularisers import FGP_TV

    vols = _volumes(shapes, 5)
    lams = [0.03 + 0.01 * i for i in range(len(vols))]
    # a single 2D call with an even row length runs the two-pixel kernel; the
    # batch runs the one-voxel kernel's arithmetic
    monkeypatch.setenv("CILREG_FGP_KERNEL", "stream")
    for graph in ("1", "0"):
        monkeypatch.setenv("CILREG_BATCH_GRAPH", graph)
        infos = np.zeros((len(vols), 2), np.float32)
        outs = FGP_TV_batch(vols, lams, 60, epsil, 0, 1, infovectors=infos)
        for v, o, lam, inf in zip(vols, outs, lams, infos):
            ref_info = np.zeros(2, np.float32)
            ref = FGP_TV(v, lam, 60, epsil, 0, 1, device="gpu", infovector=ref_info)
            assert int(inf[0]) == int(ref_info[0])
            np.testing.assert_array_equal(o, ref)


@pytest.mark.parametrize("shapes", [SHAPES_3D, SHAPES_2D], ids=["3d", "2d"])
@pytest.mark.parametrize("epsil", [0.0, 3e-3])
def test_tgv_batch_equals_single_calls(shapes, epsil):
    from ccpi.filters.batch import TGV_batch
    from ccpi.filters.regularisers import TGV

    vols = _volumes(shapes, 6)
    infos = np.zeros((len(vols), 2), np.float32)
    outs = TGV_batch(vols, 0.05, 1.0, 2.0, 40, 12.0, epsil, infovectors=infos)
    for v, o, inf in zip(vols, outs, infos):
        ref_info = np.zeros(2, np.float32)
        ref = TGV(v, 0.05, 1.0, 2.0, 40, 12.0, epsil, device="gpu", infovector=ref_info)
        assert int(inf[0]) == int(ref_info[0])
        # same arithmetic; the compiler may contract multiply-adds differently in
        # the batched instantiation, so agreement is to the last bits
        assert np.max(np.abs(o - ref)) <= rel_tol(ref, 1e-6)


SHAPES_3D_X4 = [(17, 30, 40), (64, 33, 20), (9, 9, 72), (40, 40, 40), (3, 200, 32), (70, 12, 4)]


@pytest.mark.parametrize("epsil", [0.0, 3e-3])
def test_tgv_batch_with_tensor_copy_staging(epsil, monkeypatch):
    """Every x extent a multiple of 4: the batch stages its inputs by tensor
    copies and agrees with the thread-loading batch and with single calls
    (the same stopping iterations)."""
    from ccpi.filters.batch import TGV_batch
    from ccpi.filters.regularisers import TGV

    vols = _volumes(SHAPES_3D_X4, 8)
    infos = np.zeros((len(vols), 2), np.float32)
    outs = TGV_batch(vols, 0.05, 1.0, 2.0, 40, 12.0, epsil, infovectors=infos)
    monkeypatch.setenv("CILREG_TGV_TMA", "0")
    infos0 = np.zeros((len(vols), 2), np.float32)
    outs0 = TGV_batch(vols, 0.05, 1.0, 2.0, 40, 12.0, epsil, infovectors=infos0)
    monkeypatch.delenv("CILREG_TGV_TMA")
    np.testing.assert_array_equal(infos[:, 0], infos0[:, 0])
    for v, o, o0, inf in zip(vols, outs, outs0, infos):
        assert np.max(np.abs(o - o0)) <= rel_tol(o0, 1e-6)
        ref_info = np.zeros(2, np.float32)
        ref = TGV(v, 0.05, 1.0, 2.0, 40, 12.0, epsil, device="gpu", infovector=ref_info)
        assert int(inf[0]) == int(ref_info[0])
        assert np.max(np.abs(o - ref)) <= rel_tol(ref, 1e-6)


def test_fgp_batch_autotuned_chunks(monkeypatch, tmp_path):
    """Any z chunk the autotuner picks computes the same iteration."""
    import torch
    from ccpi.filters.batch import FGP_TV_batch

    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("CILREG_BATCH_AUTOTUNE", "1")
    monkeypatch.setenv("CILREG_AUTOTUNE_CACHE", str(cache))
    vols = [torch.from_numpy(v).cuda() for v in _volumes([(96, 64, 80), (130, 40, 33)], 7)]
    a = FGP_TV_batch(vols, 0.03, 30)
    assert cache.exists() and cache.read_text().count("\t") == 1
    monkeypatch.setenv("CILREG_BATCH_AUTOTUNE", "0")
    b = FGP_TV_batch(vols, 0.03, 30)
    for x, y in zip(a, b):
        assert torch.max(torch.abs(x - y)).item() <= rel_tol(y.cpu().numpy(), 1e-6)


@pytest.mark.parametrize("shapes", [SHAPES_3D, SHAPES_2D], ids=["3d", "2d"])
@pytest.mark.parametrize("epsil", [0.0, 3e-4])
@pytest.mark.parametrize("mode", ["persistent", "persistent:1"], ids=["one-group", "l2-groups"])
def test_fgp_persistent_batch_equals_single_calls(shapes, epsil, mode, monkeypatch):
    """The persistent kernel (every iteration of every volume in one launch,
    per-volume dependency waits; with 1 MB groups, one volume after another)
    gives the single-call results bit for bit and the same stopping
    iterations."""
    from ccpi.filters.batch import FGP_TV_batch
    from ccpi.filters.regularisers import FGP_TV

    vols = _volumes(shapes, 9)
    lams = [0.03 + 0.01 * i for i in range(len(vols))]
    monkeypatch.setenv("CILREG_BATCH_MODE", mode)
    monkeypatch.setenv("CILREG_FGP_KERNEL", "stream")  # the batch's one-voxel arithmetic in 2D too
    infos = np.zeros((len(vols), 2), np.float32)
    outs = FGP_TV_batch(vols, lams, 60, epsil, 0, 1, infovectors=infos)
    for v, o, lam, inf in zip(vols, outs, lams, infos):
        ref_info = np.zeros(2, np.float32)
        ref = FGP_TV(v, lam, 60, epsil, 0, 1, device="gpu", infovector=ref_info)
        assert int(inf[0]) == int(ref_info[0])
        np.testing.assert_array_equal(o, ref)


def test_fgp_persistent_batch_on_the_seeded_batch_equals_graph(monkeypatch):
    """Sixteen uneven volumes of the seeded batch, 40 iterations: the
    persistent schedule (one group and 96 MB groups) equals the graph of
    flat-grid launches bit for bit."""
    import torch
    from ccpi.filters.batch import FGP_TV_batch

    rng = np.random.default_rng(2)
    shapes = rng.choice([96, 128, 160, 192, 256], size=(16, 3))
    vols = [torch.from_numpy(v).cuda() for v in _volumes([tuple(int(e) for e in sh) for sh in shapes], 4)]
    monkeypatch.setenv("CILREG_BATCH_MODE", "graph")
    ref = FGP_TV_batch(vols, 0.03, 40, 0.0, 0, 1)
    for mode in ("persistent", "persistent:96"):
        monkeypatch.setenv("CILREG_BATCH_MODE", mode)
        got = FGP_TV_batch(vols, 0.03, 40, 0.0, 0, 1)
        for a, b in zip(got, ref):
            assert torch.equal(a, b), mode


@pytest.mark.parametrize("epsil", [0.0, 3e-4])
def test_fgp_two_voxel_batch_equals_one_voxel_batch(epsil, monkeypatch):
    """Every x extent even: the graph of two-voxel launches agrees with the
    graph of one-voxel launches to the last bits (the paired instructions
    round each product and sum once, as the one-voxel code does) and stops
    at the same iterations."""
    from ccpi.filters.batch import FGP_TV_batch

    vols = _volumes(SHAPES_3D_X4, 10)
    lams = [0.03 + 0.01 * i for i in range(len(vols))]
    runs = {}
    for mode in ("graph", "x2"):
        monkeypatch.setenv("CILREG_BATCH_MODE", mode)
        infos = np.zeros((len(vols), 2), np.float32)
        runs[mode] = (FGP_TV_batch(vols, lams, 60, epsil, 0, 1, infovectors=infos), infos)
    (ref, ref_info), (got, got_info) = runs["graph"], runs["x2"]
    np.testing.assert_array_equal(got_info[:, 0], ref_info[:, 0])
    for a, b in zip(got, ref):
        assert np.max(np.abs(a - b)) <= rel_tol(b, 1e-5)


def test_fgp_two_voxel_batch_equals_single_calls(monkeypatch):
    """Volumes of 2^21 voxels and more, where a single call runs the
    two-voxel kernel too: the batch gives its results bit for bit, whatever
    the z chunks of the two runs."""
    import torch
    from ccpi.filters.batch import FGP_TV_batch
    from ccpi.filters.regularisers import FGP_TV

    vols = [torch.from_numpy(v).cuda() for v in _volumes([(40, 231, 230), (33, 250, 258)], 11)]
    monkeypatch.setenv("CILREG_BATCH_MODE", "x2")
    got = FGP_TV_batch(vols, [0.03, 0.05], 30, 0.0, 0, 1)
    for v, lam, o in zip(vols, (0.03, 0.05), got):
        ref = FGP_TV(v.cpu().numpy(), lam, 30, 0.0, 0, 1, device="gpu")
        np.testing.assert_array_equal(o.cpu().numpy(), ref)


@pytest.mark.parametrize("epsil", [0.0, 3e-4])
def test_fgp_2d_batch_with_even_rows_equals_single_calls(epsil):
    """2D images whose rows all have an even length: single calls run the
    two-pixel kernel, and so does the batch (its 2D tile), so the batch gives
    the single-call results bit for bit, with the same stopping iterations."""
    from ccpi.filters.batch import FGP_TV_batch
    from ccpi.filters.regularisers import FGP_TV

    vols = _volumes([(37, 52), (128, 10), (200, 200), (1, 78), (300, 2)], 12)
    lams = [0.03 + 0.01 * i for i in range(len(vols))]
    infos = np.zeros((len(vols), 2), np.float32)
    outs = FGP_TV_batch(vols, lams, 60, epsil, 0, 1, infovectors=infos)
    for v, o, lam, inf in zip(vols, outs, lams, infos):
        ref_info = np.zeros(2, np.float32)
        ref = FGP_TV(v, lam, 60, epsil, 0, 1, device="gpu", infovector=ref_info)
        assert int(inf[0]) == int(ref_info[0])
        np.testing.assert_array_equal(o, ref)


def test_batch_rejects_mixed_dimensionality():
    from ccpi.filters.batch import FGP_TV_batch

    with pytest.raises(ValueError):
        FGP_TV_batch(_volumes([(8, 8), (4, 8, 8)], 1), 0.05, 5)
