"""Prox sessions and the continuous-batching server: a request's result is the
same alone and in a concurrent mix; admission respects the HBM budget; a cold
session's first prox equals the plain call."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(n, seed, spacing=0.004):
    from ccpi.filters.serving import ProxRequest

    rng = np.random.default_rng(seed)
    algs = [("ROF", (0.02, 0.001)), ("FGP", (0.05, 0, 1)), ("SB", (0.05, 0)), ("NDF", (0.02, 0.02, 0.01, 1))]
    reqs = []
    for i in range(n):
        alg, prm = algs[i % 4]
        shape = (48, 64) if i % 3 == 0 else (16, 20, 24)
        vol = rng.random(shape).astype(np.float32)
        reqs.append(ProxRequest(i, alg, vol, prm, outer=int(rng.integers(2, 6)), inner=7,
                                arrival=spacing * i))
    return reqs


def test_result_same_alone_and_in_the_mix():
    import torch
    from ccpi.filters.serving import ProxServer, run_one

    reqs = _requests(12, 1, spacing=0.0)  # a burst: four requests start together
    mixed = ProxServer(slots=4).serve(reqs)
    s = torch.cuda.Stream()
    for r, got in zip(reqs, mixed):
        alone = run_one(r, s)
        np.testing.assert_array_equal(got.output, alone)
    # requests really overlapped: some started before an earlier one ended
    spans = sorted((m.start, m.end) for m in mixed)
    assert any(b[0] < a[1] for a, b in zip(spans, spans[1:]))


def test_admission_serialises_under_a_small_budget():
    from ccpi.filters.serving import ProxServer, request_bytes

    reqs = _requests(6, 2)
    budget = max(request_bytes(r) for r in reqs)
    res = ProxServer(slots=4, hbm_budget=budget).serve(reqs)
    spans = sorted((m.start, m.end) for m in res)
    # with room for one request at a time no two runs overlap
    assert all(b[0] >= a[1] - 1e-4 for a, b in zip(spans, spans[1:]))
    ref = ProxServer(slots=1).serve(reqs, realtime=False)
    for a, b in zip(res, ref):
        np.testing.assert_array_equal(a.output, b.output)


def test_oversize_request_is_refused():
    from ccpi.filters.serving import ProxServer

    with pytest.raises(ValueError):
        ProxServer(slots=2, hbm_budget=1000).serve(_requests(1, 3))


@pytest.mark.parametrize("alg, prm", [(0, (0.02, 0.001)), (1, (0.05, 0, 1)), (2, (0.05, 0)),
                                      (3, (0.02, 0.02, 0.01, 1))])
def test_cold_session_prox_equals_plain_call_and_state_persists(alg, prm):
    import ctypes

    import torch
    from ccpi.filters import regularisersCuPy as D
    from ccpi.filters.utils import check_status, cilregcuda

    x = torch.from_numpy(np.random.default_rng(alg).random((12, 20, 26)).astype(np.float32)).cuda()
    plain = {0: lambda: D.ROF_TV(x, prm[0], 9, prm[1]), 1: lambda: D.FGP_TV(x, prm[0], 9, 0.0, prm[1], prm[2]),
             2: lambda: D.SB_TV(x, prm[0], 9, 0.0, prm[1]),
             3: lambda: D.NDF(x, prm[0], prm[1], 9, prm[2], prm[3])}[alg]()
    sess = ctypes.c_void_p()
    p = (ctypes.c_float * 4)(*(list(prm) + [0.0] * (4 - len(prm))))
    h = torch.cuda.current_stream().cuda_stream
    check_status(cilregcuda.cilreg_prox_session_create(ctypes.byref(sess), alg, p, len(prm), 26, 20, 12, h))
    try:
        out1 = torch.zeros_like(x)
        out2 = torch.zeros_like(x)
        check_status(cilregcuda.cilreg_prox_session_prox(sess, x.data_ptr(), out1.data_ptr(), 9, 0.0, None, h))
        check_status(cilregcuda.cilreg_prox_session_prox(sess, x.data_ptr(), out2.data_ptr(), 9, 0.0, None, h))
    finally:
        cilregcuda.cilreg_prox_session_destroy(sess, h)
    torch.cuda.synchronize()
    assert torch.equal(out1, plain)
    assert not torch.equal(out2, out1)  # the second prox started from the kept state
