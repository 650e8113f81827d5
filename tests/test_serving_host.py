"""Host-side fault injection for the prox server (no GPU): the scheduling,
admission, failure isolation and cancellation logic of ProxServer with a fake
runner in place of the device solve.  A worker that raises, a request that
can never fit the budget, and requests cancelled while waiting or while
running each get their own result; every other request completes."""
import threading
import time

import numpy as np
import pytest


def _req(rid, size=10, arrival=0.0, outer=3):
    from ccpi.filters.serving import ProxRequest

    return ProxRequest(rid, "FGP", np.full((2, 2, size), rid, np.float32), (0.03, 0, 1), outer=outer, inner=4,
                       arrival=arrival)


def _echo_runner(log=None, delay=0.01):
    def run(req, slot, flag):
        if log is not None:
            log.append(("start", req.rid, time.perf_counter()))
        time.sleep(delay)
        if log is not None:
            log.append(("end", req.rid, time.perf_counter()))
        return req.volume * 2.0
    return run


def _sizer(req):
    return req.volume.size


def test_worker_exception_fails_only_its_request():
    from ccpi.filters.serving import ProxServer

    base = _echo_runner()

    def run(req, slot, flag):
        if req.rid == 2:
            raise RuntimeError("injected worker failure")
        return base(req, slot, flag)

    res = ProxServer(slots=3, runner=run, sizer=_sizer).serve([_req(i) for i in range(6)], realtime=False)
    assert [r.rid for r in res] == list(range(6))
    assert res[2].status == "failed" and "injected worker failure" in res[2].error and res[2].output is None
    for r in res:
        if r.rid != 2:
            assert r.ok and np.array_equal(r.output, np.full((2, 2, 10), 2.0 * r.rid, np.float32))


def test_native_error_status_is_a_failed_result():
    from ccpi.filters.serving import ProxServer
    from ccpi.filters.utils import RegulariserError

    def run(req, slot, flag):
        if req.rid == 1:
            raise RegulariserError(-4, "scratch allocation failed: injected failure")
        return req.volume

    res = ProxServer(slots=2, runner=run, sizer=_sizer).serve([_req(i) for i in range(4)], realtime=False)
    assert res[1].status == "failed" and "status -4" in res[1].error
    assert all(r.ok for r in res if r.rid != 1)


def test_request_over_the_budget_is_refused_alone():
    from ccpi.filters.serving import ProxServer

    reqs = [_req(0), _req(1, size=1000), _req(2)]
    res = ProxServer(slots=2, hbm_budget=100, runner=_echo_runner(), sizer=_sizer).serve(reqs, realtime=False)
    assert res[1].status == "refused" and "budget" in res[1].error
    assert res[0].ok and res[2].ok


def test_unknown_regulariser_is_refused_alone():
    from ccpi.filters.serving import ProxServer

    reqs = [_req(0), _req(1)]
    reqs[1].alg = "TNV"

    def sizer(req):
        if req.alg != "FGP":
            raise ValueError(f"unknown regulariser {req.alg}")
        return req.volume.size

    res = ProxServer(slots=2, runner=_echo_runner(), sizer=sizer).serve(reqs, realtime=False)
    assert res[1].status == "refused" and "TNV" in res[1].error and res[0].ok


def test_admission_keeps_within_the_budget():
    from ccpi.filters.serving import ProxServer

    lock = threading.Lock()
    live = {"bytes": 0, "max": 0}

    def run(req, slot, flag):
        with lock:
            live["bytes"] += req.volume.size
            live["max"] = max(live["max"], live["bytes"])
        time.sleep(0.02)
        with lock:
            live["bytes"] -= req.volume.size
        return req.volume

    reqs = [_req(i, size=10 + 5 * (i % 3)) for i in range(9)]
    budget = 2 * 4 * 20  # room for about two requests at a time
    res = ProxServer(slots=8, hbm_budget=budget, runner=run, sizer=_sizer).serve(reqs, realtime=False)
    assert all(r.ok for r in res)
    assert live["max"] <= budget


def test_cancel_a_waiting_request_never_starts_it():
    from ccpi.filters.serving import ProxServer

    gate = threading.Event()
    started = []

    def run(req, slot, flag):
        started.append(req.rid)
        if req.rid == 0:
            gate.wait(5)
        return req.volume

    server = ProxServer(slots=1, runner=run, sizer=_sizer)
    out = {}
    t = threading.Thread(target=lambda: out.update(res=server.serve([_req(0), _req(1), _req(2)], realtime=False)))
    t.start()
    deadline = time.time() + 5
    while 0 not in started and time.time() < deadline:
        time.sleep(0.005)
    server.cancel(1)
    gate.set()
    t.join(10)
    res = out["res"]
    assert res[1].status == "cancelled" and 1 not in started
    assert res[0].ok and res[2].ok


def test_cancel_a_running_request_stops_it():
    from ccpi.filters.serving import ProxServer
    from ccpi.filters.utils import RegulariserError

    running = threading.Event()

    def run(req, slot, flag):
        if req.rid == 0:
            running.set()
            for _ in range(500):  # outer steps: the native loop reads the flag before each
                if flag.value:
                    raise RegulariserError(-5, "cancelled")
                time.sleep(0.01)
            return req.volume
        return req.volume

    server = ProxServer(slots=2, runner=run, sizer=_sizer)
    out = {}
    t = threading.Thread(target=lambda: out.update(res=server.serve([_req(0), _req(1)], realtime=False)))
    t.start()
    assert running.wait(5)
    server.cancel(0)
    t.join(10)
    res = out["res"]
    assert res[0].status == "cancelled" and res[0].output is None
    assert res[1].ok


def test_summary_counts_outcomes():
    from ccpi.filters.serving import ProxResult, summarise

    rs = [ProxResult(0, np.zeros(1), 0.0, 0.0, 1.0, 8, 10), ProxResult(1, None, 0.0, 0.0, 0.5, 8, 0, "failed", "x"),
          ProxResult(2, None, 0.0, 0.0, 0.1, 8, 0, "cancelled")]
    s = summarise(rs, 2.0)
    assert (s["completed"], s["failed"], s["cancelled"]) == (1, 1, 1)
    assert s["requests_per_s"] == pytest.approx(0.5)
