"""Continuous-batching server for prox / denoising requests on one GPU.

Each request asks for ``min_x 1/2 ||w^(1/2)(x - f)||^2 + R(x)`` with R one of
ROF-TV, FGP-TV, SB-TV or NDF, solved by ``outer`` steps of FISTA, ADMM or
PDHG whose proxes are ``inner`` warm-started regulariser iterations; the
regulariser's dual / Bregman state stays on the device for the whole solve (a
native prox session, ``cilreg_prox_session_*``).

Scheduling: requests are admitted in arrival order as soon as a slot is free
and their device footprint (``cilreg_prox_session_bytes`` plus input and
output) fits in the HBM budget; a request that arrives while others run
starts at once on its own CUDA stream, so the work of all admitted requests
overlaps on the device.  Results are independent of the mix: every request's
kernels read only its own buffers.

Failure isolation: every request gets its own ProxResult.  A request that
cannot ever fit the budget is refused, one whose solve fails (a native error
status, an exception in its worker) is reported failed with the message, and
one cancelled with ``ProxServer.cancel`` before or while it runs is reported
cancelled; the other requests are served as if it had not been there.  The
reference has no serving layer: its GPU entry points print an error and
return -1 (src/Core/regularisers_GPU/shared.h:15-38), which its Python layer
ignores.
"""
from __future__ import annotations

import ctypes
import threading
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from .utils import RegulariserError, check_status, cilregcuda

ALGORITHMS = {"ROF": 0, "FGP": 1, "SB": 2, "NDF": 3}
SOLVERS = ("fista", "admm", "pdhg")
CANCELLED = -5


@dataclass
class ProxRequest:
    rid: int
    alg: str                 # "ROF", "FGP", "SB" or "NDF"
    volume: np.ndarray       # float32, (Y, X) or (Z, Y, X)
    params: tuple            # ROF (lambda, tau); FGP (lambda, methodTV, nonneg); SB (mu, methodTV);
                             # NDF (lambda, sigma, tau, penalty)
    outer: int = 10          # outer steps
    inner: int = 20          # regulariser iterations per prox
    step: float = 0.5        # FISTA gradient step on 1/2 ||x - f||^2
    arrival: float = 0.0     # seconds after the start of the stream
    solver: str = "fista"    # "fista", "admm" (penalty rho) or "pdhg" (steps tau, sigma)
    rho: float = 1.0
    tau: float = 1.0
    sigma: float = 1.0
    weights: Optional[np.ndarray] = None  # ADMM / PDHG per-voxel data weights (None: all ones)


@dataclass
class ProxResult:
    rid: int
    output: Optional[np.ndarray]
    arrival: float
    start: float
    end: float
    voxels: int
    iterations: int
    status: str = "ok"       # "ok", "failed", "refused" or "cancelled"
    error: Optional[str] = None
    latency: float = field(init=False)

    def __post_init__(self):
        self.latency = self.end - self.arrival

    @property
    def ok(self) -> bool:
        return self.status == "ok"


def _dims(shape):
    d = list(shape)[::-1]
    if len(shape) == 2:
        d.append(1)
    return d


def request_bytes(req: ProxRequest) -> int:
    """Device bytes a request holds while admitted (session + input + output,
    + weights)."""
    if req.alg not in ALGORITHMS:
        raise ValueError(f"request {req.rid}: unknown regulariser {req.alg!r}")
    b = int(cilregcuda.cilreg_prox_session_bytes(ALGORITHMS[req.alg], *_dims(req.volume.shape)))
    if b < 0:
        raise ValueError(f"bad request {req.rid}")
    extra = 4 * req.volume.size if req.weights is not None else 0
    return b + 2 * 4 * req.volume.size + extra


def run_one(req: ProxRequest, stream, cancel_flag: Optional[ctypes.c_int] = None) -> np.ndarray:
    """Solve one request on `stream` (a torch.cuda.Stream).  With `cancel_flag`
    the native loop reads it before every outer step and stops with status -5
    (RegulariserError) once it is nonzero."""
    import torch

    if req.solver not in SOLVERS:
        raise ValueError(f"request {req.rid}: unknown solver {req.solver!r}")
    with torch.cuda.stream(stream):
        f = torch.from_numpy(np.ascontiguousarray(req.volume, dtype=np.float32)).pin_memory().to(
            "cuda", non_blocking=True)
        w = None
        if req.weights is not None:
            w = torch.from_numpy(np.ascontiguousarray(req.weights, dtype=np.float32)).to("cuda", non_blocking=True)
            if w.shape != f.shape:
                raise ValueError(f"request {req.rid}: weights of shape {tuple(w.shape)} for a volume {tuple(f.shape)}")
        x = torch.empty_like(f)
        params = (ctypes.c_float * 4)(*[float(p) for p in req.params] + [0.0] * (4 - len(req.params)))
        sess = ctypes.c_void_p()
        h = stream.cuda_stream
        check_status(cilregcuda.cilreg_prox_session_create(ctypes.byref(sess), ALGORITHMS[req.alg], params,
                                                           len(req.params), *_dims(req.volume.shape), h))
        try:
            if cancel_flag is not None:
                check_status(cilregcuda.cilreg_prox_session_set_cancel(sess, ctypes.byref(cancel_flag)))
            wp = w.data_ptr() if w is not None else None
            if req.solver == "fista":
                st = cilregcuda.cilreg_prox_session_fista(sess, f.data_ptr(), x.data_ptr(), int(req.outer),
                                                          int(req.inner), float(req.step), h)
            elif req.solver == "admm":
                st = cilregcuda.cilreg_prox_session_admm(sess, f.data_ptr(), wp, x.data_ptr(), int(req.outer),
                                                         int(req.inner), float(req.rho), h)
            else:
                st = cilregcuda.cilreg_prox_session_pdhg(sess, f.data_ptr(), wp, x.data_ptr(), int(req.outer),
                                                         int(req.inner), float(req.tau), float(req.sigma), h)
            check_status(st)
        finally:
            cilregcuda.cilreg_prox_session_destroy(sess, h)
        out = x.cpu()
    return out.numpy()


class ProxServer:
    """Admit requests as slots and HBM free up; run admitted requests concurrently.

    `runner(req, slot, cancel_flag)` solves one request (default: `run_one` on
    the slot's CUDA stream); `sizer(req)` gives its device bytes (default:
    `request_bytes`).  Both are replaceable so that the scheduling, isolation
    and cancellation logic can be exercised without a GPU."""

    def __init__(self, slots: int = 8, hbm_budget: float = 150e9, device: int = 0,
                 runner: Optional[Callable] = None, sizer: Optional[Callable] = None):
        self.slots = slots
        self.budget = int(hbm_budget)
        self.device = device
        self.sizer = sizer or request_bytes
        self._cancel_lock = threading.Lock()
        self._cancelled = set()
        self._flags = {}
        if runner is None:
            import torch

            torch.cuda.set_device(device)
            streams = [torch.cuda.Stream(device) for _ in range(slots)]

            def runner(req, slot, flag):
                torch.cuda.set_device(self.device)
                return run_one(req, streams[slot], flag)

        self.runner = runner

    def cancel(self, rid: int) -> None:
        """Cancel request `rid`: it is not started if still waiting, and a
        running solve stops before its next outer step."""
        with self._cancel_lock:
            self._cancelled.add(rid)
            flag = self._flags.get(rid)
            if flag is not None:
                flag.value = 1

    def serve(self, requests, realtime: bool = True):
        """Serve `requests` (their .arrival times relative to now when realtime);
        return one ProxResult per request, ordered by request id."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        lock = threading.Condition()
        pending = deque()
        free_slots = list(range(self.slots))
        state = {"in_use": 0, "done": 0}
        results = {}
        sizes = {}
        t0 = time.perf_counter()

        def finish(req, start, status, out=None, error=None):
            end = time.perf_counter() - t0
            results[req.rid] = ProxResult(req.rid, out, req.arrival, start, end, req.volume.size,
                                          req.outer * req.inner if status == "ok" else 0, status, error)

        def worker(req, slot, nbytes, start):
            flag = ctypes.c_int(0)
            with self._cancel_lock:
                self._flags[req.rid] = flag
                if req.rid in self._cancelled:
                    flag.value = 1
            try:
                if flag.value:
                    finish(req, start, "cancelled")
                else:
                    out = self.runner(req, slot, flag)
                    finish(req, start, "ok", out)
            except RegulariserError as exc:
                finish(req, start, "cancelled" if exc.status == CANCELLED else "failed", error=str(exc))
            except Exception as exc:  # the request fails, the server keeps serving
                finish(req, start, "failed", error=f"{type(exc).__name__}: {exc}")
            with self._cancel_lock:
                self._flags.pop(req.rid, None)
            with lock:
                state["in_use"] -= nbytes
                state["done"] += 1
                free_slots.append(slot)
                lock.notify_all()

        def admit_locked():
            while pending and free_slots:
                req = pending[0]
                with self._cancel_lock:
                    gone = req.rid in self._cancelled
                if gone:  # cancelled while waiting: never started
                    pending.popleft()
                    now = time.perf_counter() - t0
                    finish(req, now, "cancelled")
                    state["done"] += 1
                    continue
                nbytes = sizes[req.rid]
                if state["in_use"] + nbytes > self.budget:
                    break  # wait for memory to free up, in arrival order
                pending.popleft()
                slot = free_slots.pop()
                state["in_use"] += nbytes
                start = time.perf_counter() - t0
                threading.Thread(target=worker, args=(req, slot, nbytes, start), daemon=True).start()

        for req in reqs:
            with lock:
                # until this request arrives, admit pending ones as completions free room
                while realtime:
                    delay = req.arrival - (time.perf_counter() - t0)
                    if delay <= 0:
                        break
                    lock.wait(timeout=delay)
                    admit_locked()
                try:
                    sizes[req.rid] = int(self.sizer(req))
                    refused = None if sizes[req.rid] <= self.budget else "needs more than the HBM budget"
                except Exception as exc:  # unknown regulariser, bad shape
                    refused = f"{type(exc).__name__}: {exc}"
                if refused is not None:
                    now = time.perf_counter() - t0
                    finish(req, now, "refused", error=f"request {req.rid}: {refused}")
                    state["done"] += 1
                else:
                    pending.append(req)
                admit_locked()
        with lock:
            while state["done"] < len(reqs):
                admit_locked()
                lock.wait(timeout=0.05)
        return [results[r.rid] for r in sorted(reqs, key=lambda r: r.rid)]


def summarise(results, wall: float):
    done = [r for r in results if r.ok]
    lat = np.array([r.latency for r in done]) if done else np.zeros(1)
    vox_it = sum(r.voxels * r.iterations for r in done)
    return {"requests": len(results), "completed": len(done), "failed": sum(r.status == "failed" for r in results),
            "refused": sum(r.status == "refused" for r in results),
            "cancelled": sum(r.status == "cancelled" for r in results), "wall_s": wall,
            "requests_per_s": len(done) / wall,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_latency_s": float(lat.mean()), "voxel_iters_per_s": vox_it / wall}
