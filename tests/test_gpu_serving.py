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

    res = ProxServer(slots=2, hbm_budget=1000).serve(_requests(1, 3))
    assert res[0].status == "refused" and res[0].output is None


def test_injected_allocation_failure_fails_one_request_only():
    """The library's next device allocation fails (host-side injection): the
    request that made it gets a failed result with the out-of-memory status,
    every other request equals its result alone."""
    import torch
    from ccpi.filters.serving import ProxServer, run_one
    from ccpi.filters.utils import cilregcuda

    reqs = _requests(8, 4, spacing=0.0)
    server = ProxServer(slots=1)  # one at a time: the first allocation belongs to request 0
    cilregcuda.cilreg_debug_fail_allocations(1)
    try:
        res = server.serve(reqs, realtime=False)
    finally:
        cilregcuda.cilreg_debug_fail_allocations(0)
    failed = [r for r in res if r.status == "failed"]
    assert len(failed) == 1 and "status -4" in failed[0].error, [(r.rid, r.status, r.error) for r in res]
    s = torch.cuda.Stream()
    for r, got in zip(reqs, res):
        if got.ok:
            np.testing.assert_array_equal(got.output, run_one(r, s))


def test_cancel_a_running_solve_on_the_device():
    import threading
    import time

    from ccpi.filters.serving import ProxRequest, ProxServer

    # about 3000 x 20 FGP iterations of 10.5 M voxels: several seconds uncancelled
    big = ProxRequest(0, "FGP", np.random.default_rng(0).random((160, 256, 256)).astype(np.float32), (0.03, 0, 1),
                      outer=3000, inner=20)
    small = _requests(3, 5, spacing=0.0)
    for i, r in enumerate(small):
        r.rid = i + 1
    server = ProxServer(slots=4)
    out = {}
    t = threading.Thread(target=lambda: out.update(res=server.serve([big] + small, realtime=False)))
    t0 = time.perf_counter()
    t.start()
    time.sleep(0.5)
    server.cancel(0)
    t.join(120)
    res = out["res"]
    assert res[0].status == "cancelled" and res[0].output is None
    assert all(r.ok for r in res[1:])
    assert time.perf_counter() - t0 < 4.0  # the whole solve would take longer


@pytest.mark.parametrize("solver", ["admm", "pdhg"])
@pytest.mark.parametrize("alg, name, prm", [(1, "FGP", (0.03, 0, 1)), (2, "SB", (0.03, 0)), (0, "ROF", (0.02, 0.001)),
                                            (3, "NDF", (0.02, 0.02, 0.01, 1))], ids=["FGP", "SB", "ROF", "NDF"])
@pytest.mark.parametrize("weighted", [False, True], ids=["w1", "mask"])
def test_admm_pdhg_against_oracle(solver, alg, name, prm, weighted):
    """ADMM and PDHG outer loops over a warm prox session (7 outer steps of 15
    inner iterations) against the oracle's loops over the port's warm proxes;
    with unit weights and with a 0/1 inpainting mask."""
    import torch
    from ccpi.filters.serving import ProxRequest, run_one
    from ccpi.supp.phantoms import noisy_phantom

    import oracle as O
    from conftest import rel_tol

    f = noisy_phantom((24, 40, 48), 8, 11 + alg)
    w = (np.random.default_rng(alg).random(f.shape) > 0.3).astype(np.float32) if weighted else None
    req = ProxRequest(0, name, f, prm, outer=7, inner=15, solver=solver, rho=1.5, tau=0.8, sigma=1.25, weights=w)
    out = run_one(req, torch.cuda.Stream())
    if solver == "admm":
        ref = O.admm(alg, f, prm, 7, 15, 1.5, w)
    else:
        ref = O.pdhg(alg, f, prm, 7, 15, 0.8, 1.25, w)
    err = float(np.max(np.abs(out - ref)))
    assert err <= rel_tol(ref, 1e-4), err


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
