"""Continuous-batching server for prox / denoising requests on one GPU.

Each request asks for ``min_x 1/2 ||x - f||^2 + R(x)`` with R one of ROF-TV,
FGP-TV, SB-TV or NDF, solved by ``outer`` FISTA steps whose proxes are
``inner`` warm-started regulariser iterations; the regulariser's dual /
Bregman state stays on the device for the whole solve (a native prox session,
``cilreg_prox_session_*``).

Scheduling: requests are admitted in arrival order as soon as a slot is free
and their device footprint (``cilreg_prox_session_bytes`` plus input and
output) fits in the HBM budget; a request that arrives while others run
starts at once on its own CUDA stream, so the work of all admitted requests
overlaps on the device.  Results are independent of the mix: every request's
kernels read only its own buffers.
"""
from __future__ import annotations

import ctypes
import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .utils import check_status, cilregcuda

ALGORITHMS = {"ROF": 0, "FGP": 1, "SB": 2, "NDF": 3}


@dataclass
class ProxRequest:
    rid: int
    alg: str                 # "ROF", "FGP", "SB" or "NDF"
    volume: np.ndarray       # float32, (Y, X) or (Z, Y, X)
    params: tuple            # ROF (lambda, tau); FGP (lambda, methodTV, nonneg); SB (mu, methodTV);
                             # NDF (lambda, sigma, tau, penalty)
    outer: int = 10          # FISTA steps
    inner: int = 20          # regulariser iterations per prox
    step: float = 0.5        # FISTA gradient step on 1/2 ||x - f||^2
    arrival: float = 0.0     # seconds after the start of the stream


@dataclass
class ProxResult:
    rid: int
    output: np.ndarray
    arrival: float
    start: float
    end: float
    voxels: int
    iterations: int
    latency: float = field(init=False)

    def __post_init__(self):
        self.latency = self.end - self.arrival


def _dims(shape):
    d = list(shape)[::-1]
    if len(shape) == 2:
        d.append(1)
    return d


def request_bytes(req: ProxRequest) -> int:
    """Device bytes a request holds while admitted (session + input + output)."""
    b = int(cilregcuda.cilreg_prox_session_bytes(ALGORITHMS[req.alg], *_dims(req.volume.shape)))
    if b < 0:
        raise ValueError(f"bad request {req.rid}")
    return b + 2 * 4 * req.volume.size


def run_one(req: ProxRequest, stream) -> np.ndarray:
    """Solve one request on `stream` (a torch.cuda.Stream)."""
    import torch

    with torch.cuda.stream(stream):
        f = torch.from_numpy(np.ascontiguousarray(req.volume, dtype=np.float32)).pin_memory().to(
            "cuda", non_blocking=True)
        x = torch.empty_like(f)
        params = (ctypes.c_float * 4)(*[float(p) for p in req.params] + [0.0] * (4 - len(req.params)))
        sess = ctypes.c_void_p()
        h = stream.cuda_stream
        check_status(cilregcuda.cilreg_prox_session_create(ctypes.byref(sess), ALGORITHMS[req.alg], params,
                                                           len(req.params), *_dims(req.volume.shape), h))
        try:
            check_status(cilregcuda.cilreg_prox_session_fista(sess, f.data_ptr(), x.data_ptr(), int(req.outer),
                                                              int(req.inner), float(req.step), h))
        finally:
            cilregcuda.cilreg_prox_session_destroy(sess, h)
        out = x.cpu()
    return out.numpy()


class ProxServer:
    """Admit requests as slots and HBM free up; run admitted requests concurrently."""

    def __init__(self, slots: int = 8, hbm_budget: float = 150e9, device: int = 0):
        import torch

        self.slots = slots
        self.budget = int(hbm_budget)
        self.device = device
        torch.cuda.set_device(device)
        self.streams = [torch.cuda.Stream(device) for _ in range(slots)]

    def serve(self, requests, realtime: bool = True):
        """Serve `requests` (their .arrival times relative to now when realtime);
        return the ProxResults ordered by request id."""
        import torch

        reqs = sorted(requests, key=lambda r: r.arrival)
        for r in reqs:
            if request_bytes(r) > self.budget:
                raise ValueError(f"request {r.rid} needs more than the HBM budget")
        lock = threading.Condition()
        pending = deque()
        free_streams = list(range(self.slots))
        state = {"in_use": 0, "done": 0, "error": None}
        results = {}
        t0 = time.perf_counter()

        def worker(req, slot, nbytes, start):
            try:
                torch.cuda.set_device(self.device)
                out = run_one(req, self.streams[slot])
                end = time.perf_counter() - t0
                results[req.rid] = ProxResult(req.rid, out, req.arrival, start, end, req.volume.size,
                                              req.outer * req.inner)
            except Exception as exc:  # the request fails, the server keeps serving
                state["error"] = exc
                results[req.rid] = None
            with lock:
                state["in_use"] -= nbytes
                state["done"] += 1
                free_streams.append(slot)
                lock.notify_all()

        def admit_locked():
            while pending and free_streams:
                req = pending[0]
                nbytes = request_bytes(req)
                if state["in_use"] + nbytes > self.budget:
                    break  # wait for memory to free up, in arrival order
                pending.popleft()
                slot = free_streams.pop()
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
                pending.append(req)
                admit_locked()
        with lock:
            while state["done"] < len(reqs):
                admit_locked()
                lock.wait(timeout=0.05)
        if state["error"] is not None:
            raise state["error"]
        return [results[r.rid] for r in sorted(reqs, key=lambda r: r.rid)]


def summarise(results, wall: float):
    lat = np.array([r.latency for r in results])
    vox_it = sum(r.voxels * r.iterations for r in results)
    return {"requests": len(results), "wall_s": wall, "requests_per_s": len(results) / wall,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_latency_s": float(lat.mean()), "voxel_iters_per_s": vox_it / wall}
