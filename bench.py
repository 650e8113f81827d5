"""Benchmark: FGP-TV 3D on a 512^3 float32 volume (voxel-iterations per second).

Workload (one "step" = one full regulariser call): the seeded 30-ellipsoid
phantom plus N(0, 0.05^2) noise at 512^3, lambda 0.03, isotropic TV,
nonnegativity on, up to 500 iterations with the stopping rule epsil = 1e-6
(the reference's stopping rule decides how many iterations run).

  value     voxel-iterations/s with input and output resident in HBM
            (device-pointer C ABI, cilreg_fgp_tv_dev), CUDA events on the stream
  e2e       the same metric through the reference-facing C ABI
            (TV_FGP_GPU_main) from pinned host buffers, copies included
  roofline  the FGP iteration kernel: 40 algorithmic bytes per voxel-iteration
            (read P^{k-1}(3), P^{k-2}(3), f; write P^k(3)) over its average
            launch time, against the measured HBM copy bandwidth
  cpu_baseline  the reference's C-OMP FGP (oracle/_ref when it is built for
            this machine, else the oracle's C restatement) on all host cores,
            a bounded sample of the same workload

Multi-GPU: one process per GPU (torchrun), each an independent replica of the
workload (the toolkit's multi-GPU model is one volume per GPU, no exchange);
value = all ranks' voxel-iterations / the slowest rank's time.

``--impl reference`` times the reference CPU implementation on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "ccpi-regularisation-toolkit_gb300")
sys.path.insert(0, PKG)

METRIC = "FGP_TV 3D voxel-iterations/s"
UNIT = "voxel-iter/s"
LAM, MAX_ITERS, EPSIL, METHOD, NONNEG = 0.03, 500, 1e-6, 0, 1
BYTES_PER_VOXEL_ITER = 40  # FGP 3D fused iteration: 7 float reads + 3 float writes


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def reduce_over_ranks(pg, t_local, units_local, device):
    """Whole-job figures of independent replicas: (slowest rank's time, sum of
    all ranks' units).  `pg` is torch.distributed (or None for one process)."""
    if pg is None:
        return float(t_local), float(units_local)
    import torch

    tt = torch.tensor([float(t_local), float(units_local)], device=device, dtype=torch.float64)
    t_max, units = tt[:1].clone(), tt[1:].clone()
    pg.all_reduce(t_max, op=pg.ReduceOp.MAX)
    pg.all_reduce(units, op=pg.ReduceOp.SUM)
    return float(t_max[0]), float(units[0])


def _phantom(size):
    from ccpi.supp.phantoms import noisy_phantom

    return noisy_phantom((size, size, size), 30, 1)


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _ncu_traffic_per_voxel():
    """DRAM bytes per voxel-iteration of the FGP kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "fgp_tv_3d_kernel.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_voxel_iter:\s*([0-9.]+)", text)
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi samples during the timed region (median SM clock, throttle reasons)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def host_info():
    """CPU model and logical core count of this host (recorded beside every CPU figure)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.split(":")[0].strip() in ("Model name", "Model"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    import platform

    return {"cpu_model": model or platform.processor() or platform.machine(), "nproc": os.cpu_count()}


def cpu_baseline(x, iters):
    """Reference C-OMP FGP on the host: the reference's own sources compiled on
    this machine (oracle/_ref) when they were staged, else the oracle's C
    restatement, with OpenMP on every host core."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    kind = "reference" if O.ref_lib() is not None else "port"
    t = time.perf_counter()
    O.fgp_tv(x, LAM, iters, 0.0, METHOD, NONNEG, use_ref=(kind == "reference"))
    dt = time.perf_counter() - t
    cores = O.num_threads()
    return x.size * iters / dt, kind, cores, dt


def run_reference(args):
    """The reference arm: the reference's CPU implementation of the path
    (TV_FGP_CPU_main, FGP_TV_core.c:40) on every host core, each step a fixed
    sample of --ref-iters iterations of the benchmark volume (epsil 0: the
    per-iteration cost is constant), reported as voxel-iterations/s."""
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    x = _phantom(args.size)
    iters = args.ref_iters
    for _ in range(args.warmup):
        cpu_baseline(x, 1)
    kind, cores, secs = None, None, 0.0
    for _ in range(args.steps):
        _, kind, cores, dt = cpu_baseline(x, iters)
        secs += dt
    value = x.size * iters * args.steps / secs
    sample = (f"FGP_TV {args.size}^3, {iters} fixed iterations per step (epsil=0; the GPU arm's per-iteration "
              f"rate is compared), iso, nonneg; warm-up steps run 1 iteration")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"FGP_TV 3D {args.size}^3 ellipsoid phantom + noise", "lambda": LAM,
                   "methodTV": "iso", "nonneg": NONNEG, "iterations_per_step": iters},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample,
                         **host_info()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def fgp_kernel_name(nx):
    """The 3D FGP iteration kernel the library runs for an x extent of nx: the
    tensor-copy-staged kernel when the row pitch allows it, else the
    thread-loading one."""
    e = os.environ.get("CILREG_FGP_TMA", "")
    if nx % 4 == 0 and e != "0" and (e == "1" or nx ** 3 >= 2 ** 25):
        return "FGP iteration (k_fgp_tma, csrc/fgp_tma.cu)"
    return "FGP iteration (k_fgp_stream, csrc/fgp_tiled.cu)"


def profile_case(args):
    """Device-only FGP calls with a fixed iteration count: the small, repeatable
    command the committed ncu summaries were captured from."""
    import ctypes

    import torch
    from ccpi.filters import utils as U

    from ccpi.filters import regularisersCuPy as D

    x = _phantom(args.size)
    d_in = torch.from_numpy(x).cuda()
    d_out = torch.zeros_like(d_in)
    info = np.zeros(2, np.float32)
    stream = torch.cuda.current_stream()
    nx = ny = nz = args.size
    others = {
        "ROF": lambda: D.ROF_TV(d_in, 0.02, args.iters, 0.001),
        "PD": lambda: D.PD_TV(d_in, 0.03, args.iters, 0.0, 0, 1, 8.0),
        "SB": lambda: D.SB_TV(d_in, 0.03, args.iters),
        "TGV": lambda: D.TGV(d_in, 0.03, 1.0, 2.0, args.iters, 12.0),
        "NDF": lambda: D.NDF(d_in, 0.02, 0.02, args.iters, 0.01, 1),
        "Diff4th": lambda: D.Diff4th(d_in, 0.8, 0.02, args.iters, 1e-4),
        "LLT_ROF": lambda: D.LLT_ROF(d_in, 0.02, 0.01, args.iters, 0.001),
        "FGP_dTV": lambda: D.FGP_dTV(d_in, d_in, 0.03, args.iters, 0.0, 0.2, 0, 1),
    }
    times = []
    for k in range(args.warmup + args.steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        if args.reg == "FGP":
            st = U.cilregcuda.cilreg_fgp_tv_dev(d_in.data_ptr(), d_out.data_ptr(),
                                                info.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), LAM, args.iters,
                                                0.0, METHOD, NONNEG, nx, ny, nz, stream.cuda_stream)
            U.check_status(st)
        else:
            others[args.reg]()
        b.record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            times.append(a.elapsed_time(b) / args.iters)
    print(json.dumps({"profile_case": f"{args.reg} 3D {args.size}^3", "iters": args.iters,
                      "ms_per_iteration": min(times)}))
    return 0


# algorithmic bytes per voxel-iteration of each regulariser's fused iteration
# algorithmic bytes per voxel-iteration (3D, 2D): each state array read and
# written once, read-only inputs read once; SB's state is U and B (D is
# recomputed from them), TGV's U, P, Q, V
SUITE_BYTES = {"ROF": (12, 12), "FGP": (40, 28), "PD": (36, 28), "SB": (36, 28), "TGV": (108, 68), "NDF": (12, 12),
               "Diff4th": (12, 12), "LLT_ROF": (12, 12), "FGP_dTV": (52, 36)}


def suite(args):
    """Per-regulariser steady-state iteration time (difference of two fixed-count
    runs on the same stream) on device-resident phantoms, with the roofline
    fraction of each against the measured HBM bandwidth."""
    import torch
    from ccpi.filters import regularisersCuPy as D
    from ccpi.supp.phantoms import noisy_phantom

    peak, peak_kind = _peaks()
    calls = {
        "ROF": lambda t, n: D.ROF_TV(t, 0.02, n, 0.001),
        "FGP": lambda t, n: D.FGP_TV(t, 0.03, n, 0.0, 0, 1),
        "PD": lambda t, n: D.PD_TV(t, 0.03, n, 0.0, 0, 1, 8.0),
        "SB": lambda t, n: D.SB_TV(t, 0.03, n),
        "TGV": lambda t, n: D.TGV(t, 0.03, 1.0, 2.0, n, 12.0),
        "NDF": lambda t, n: D.NDF(t, 0.02, 0.02, n, 0.01, 1),
        "Diff4th": lambda t, n: D.Diff4th(t, 0.8, 0.02, n, 1e-4),
        "LLT_ROF": lambda t, n: D.LLT_ROF(t, 0.02, 0.01, n, 0.001),
        "FGP_dTV": lambda t, n: D.FGP_dTV(t, t, 0.03, n, 0.0, 0.2, 0, 1),
    }
    shapes = [(256, 256, 256), (512, 512)] if args.size <= 256 else [(args.size,) * 3, (512, 512)]
    rows = []
    for shape in shapes:
        t = torch.from_numpy(noisy_phantom(shape, 30 if len(shape) == 3 else 10, 1 if len(shape) == 3 else 0)).cuda()
        n = t.numel()
        for name, fn in calls.items():
            if args.regs and name not in args.regs.split(","):
                continue
            i1, i2 = (10, 40) if len(shape) == 3 else (50, 450)

            def timed(iters):
                torch.cuda.synchronize()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record()
                fn(t, iters)
                b.record()
                torch.cuda.synchronize()
                return a.elapsed_time(b) / 1e3

            timed(i1)
            t1 = min(timed(i1) for _ in range(2))
            t2 = min(timed(i2) for _ in range(2))
            per_it = (t2 - t1) / (i2 - i1)
            bpv = SUITE_BYTES[name][0 if len(shape) == 3 else 1]
            gbs = bpv * n / per_it / 1e9
            rows.append({"regulariser": name, "shape": "x".join(map(str, shape)), "ms_per_iteration": per_it * 1e3,
                         "voxel_iters_per_s": n / per_it, "algorithmic_bytes_per_voxel_iter": bpv,
                         "achieved_gbs": gbs, "frac_of_hbm": gbs / peak})
            print(json.dumps(rows[-1]))
    print(json.dumps({"suite": rows, "peak_gbs": peak, "peak_kind": peak_kind}))
    return 0


def batch_volumes(n=64, seed=2):
    """The batched workload: n volumes, each edge drawn from {96,...,256}."""
    from ccpi.supp.phantoms import noisy_phantom

    rng = np.random.default_rng(seed)
    shapes = rng.choice([96, 128, 160, 192, 256], size=(n, 3))
    return [noisy_phantom(tuple(int(e) for e in sh), 30, 1000 + i) for i, sh in enumerate(shapes)]


def reference_gpu_lib():
    """The reference's own CUDA library (its *_GPU_main per-call path, compiled
    for sm_103a from the staged reference sources into oracle/_ref), or None
    when the sources are not staged on this machine."""
    import ctypes

    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "refgpu"], capture_output=True, text=True)
    path = os.path.join(ROOT, "oracle", "_ref", "libcilregcuda_ref.so")
    if r.returncode != 0 or not os.path.exists(path):
        return None
    lib = ctypes.CDLL(path)
    P, F, I = ctypes.POINTER(ctypes.c_float), ctypes.c_float, ctypes.c_int
    # TV_FGP_GPU_core.h:7, TGV_GPU_core.h:8, TV_ROF_GPU_core.h:6, TV_SB_GPU_core.h:8, NonlDiff_GPU_core.h:6
    lib.TV_FGP_GPU_main.argtypes = [P, P, P, F, I, F, I, I, I, I, I, I]
    lib.TGV_GPU_main.argtypes = [P, P, P, F, F, F, I, F, F, I, I, I, I]
    lib.TV_ROF_GPU_main.argtypes = [P, P, P, F, I, F, F, I, I, I, I]
    lib.TV_SB_GPU_main.argtypes = [P, P, P, F, I, F, I, I, I, I, I]
    lib.NonlDiff_GPU_main.argtypes = [P, P, P, F, F, I, F, I, F, I, I, I, I]
    for name in ("TV_FGP_GPU_main", "TGV_GPU_main", "TV_ROF_GPU_main", "TV_SB_GPU_main", "NonlDiff_GPU_main"):
        getattr(lib, name).restype = ctypes.c_int
    return lib


def reference_tgv_in_bounds(shape):
    """The reference's 3D TGV kernels index element (i, j, k) as
    (dimX*dimY)*k + i*dimX + j (TGV_GPU_core.cu:290) while TV.py:722-731 passes
    the array shape (Z, Y, X) as (dimX, dimY, dimZ); every index stays inside
    the array only when Z <= Y.  Other shapes would read and write past the
    end of the last plane, so the baseline never runs them."""
    return len(shape) == 3 and shape[0] <= shape[1]


def _ref_call(lib, name, vol, *args):
    """One per-call reference GPU run from host arrays, its dims as TV.py passes them."""
    import ctypes

    P = ctypes.POINTER(ctypes.c_float)
    a = np.ascontiguousarray(vol, dtype=np.float32)
    out = np.zeros_like(a)
    info = np.zeros(2, np.float32)
    if name == "TGV_GPU_main":
        dims = list(a.shape)  # TV.py:722-725 reverses the dims twice: (Z, Y, X)
    else:
        dims = list(a.shape)[::-1] + ([1] if a.ndim == 2 else [])
    st = getattr(lib, name)(a.ctypes.data_as(P), out.ctypes.data_as(P), info.ctypes.data_as(P), *args, 0, *dims)
    if st != 0:
        raise RuntimeError(f"reference {name} returned {st}")
    return out


def batch_bench(args):
    """Batched FGP-TV and TGV (one graph launch per regulariser) against the
    same volumes regularised one call at a time: through this library's device
    API, and through the reference's own per-call GPU path (TV_FGP_GPU_main,
    TGV_GPU_main with host arrays, as TV.py calls them).  The batched run is
    timed both on device-resident volumes and from host arrays (copies in and
    out included), the latter being the like-for-like comparison with the
    reference's host-array calls."""
    import torch
    from ccpi.filters import regularisersCuPy as D
    from ccpi.filters.batch import FGP_TV_batch, TGV_batch

    host = batch_volumes()
    vols = [torch.from_numpy(v).cuda() for v in host]
    nvox = sum(v.numel() for v in vols)
    iters = 300
    tgv_sub = [i for i, v in enumerate(host) if reference_tgv_in_bounds(v.shape)]
    runs = {
        "FGP_TV": (lambda: FGP_TV_batch(vols, 0.03, iters, 0.0, 0, 1),
                   lambda: FGP_TV_batch(host, 0.03, iters, 0.0, 0, 1),
                   lambda: [D.FGP_TV(v, 0.03, iters, 0.0, 0, 1) for v in vols],
                   list(range(len(host))),
                   lambda lib, v: _ref_call(lib, "TV_FGP_GPU_main", v, 0.03, iters, 0.0, 0, 1)),
        "TGV": (lambda: TGV_batch(vols, 0.03, 1.0, 2.0, iters, 12.0),
                lambda: TGV_batch(host, 0.03, 1.0, 2.0, iters, 12.0),
                lambda: [D.TGV(v, 0.03, 1.0, 2.0, iters, 12.0) for v in vols],
                tgv_sub,
                lambda lib, v: _ref_call(lib, "TGV_GPU_main", v, 0.03, 1.0, 2.0, iters, 12.0, 0.0)),
    }

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t

    ref = reference_gpu_lib() if not args.no_reference_gpu else None
    out = {"workload": f"{len(vols)} volumes, edges from {{96,128,160,192,256}}, {nvox} voxels, {iters} iterations",
           "results": {}}
    for name, (batched, batched_host, percall, ref_idx, ref_fn) in runs.items():
        timed(batched)
        tb = min(timed(batched) for _ in range(max(1, args.steps)))
        timed(batched_host)
        tbh = min(timed(batched_host) for _ in range(max(1, min(args.steps, 2))))
        timed(percall)
        tp = min(timed(percall) for _ in range(max(1, min(args.steps, 2))))
        r = {"batched_s": tb, "batched_from_host_s": tbh, "per_call_s": tp,
             "batched_volumes_per_s": len(vols) / tb, "batched_from_host_volumes_per_s": len(vols) / tbh,
             "per_call_volumes_per_s": len(vols) / tp, "batched_voxel_iters_per_s": nvox * iters / tb,
             "speedup_vs_per_call": tp / tb}
        if ref is not None:
            sub = [host[i] for i in ref_idx]
            sub_vox = sum(v.size for v in sub)
            _ref_call_warm = ref_fn(ref, sub[0])  # module load, context
            del _ref_call_warm
            t = time.perf_counter()
            for v in sub:
                ref_fn(ref, v)
            tr = time.perf_counter() - t
            # this library on exactly the same volumes, batched from host arrays
            sub_fn = (lambda: FGP_TV_batch(sub, 0.03, iters, 0.0, 0, 1)) if name == "FGP_TV" else \
                (lambda: TGV_batch(sub, 0.03, 1.0, 2.0, iters, 12.0))
            sub_dev = [vols[i] for i in ref_idx]
            sub_dev_fn = (lambda: FGP_TV_batch(sub_dev, 0.03, iters, 0.0, 0, 1)) if name == "FGP_TV" else \
                (lambda: TGV_batch(sub_dev, 0.03, 1.0, 2.0, iters, 12.0))
            timed(sub_fn)
            ts = min(timed(sub_fn) for _ in range(2))
            timed(sub_dev_fn)
            tsd = min(timed(sub_dev_fn) for _ in range(2))
            r["reference_per_call"] = {
                "volumes": len(sub), "voxels": sub_vox,
                "selection": ("all volumes" if len(sub) == len(host) else
                              "volumes with shape[0] <= shape[1], the only ones the reference kernels index in bounds"),
                "reference_s": tr, "reference_volumes_per_s": len(sub) / tr,
                "batched_from_host_s": ts, "batched_from_host_volumes_per_s": len(sub) / ts,
                "batched_device_s": tsd, "batched_device_volumes_per_s": len(sub) / tsd,
                "speedup_from_host": tr / ts, "speedup_device_resident": tr / tsd}
        out["results"][name] = r
        print(json.dumps({name: r}))
    if ref is None:
        out["reference_per_call"] = "unavailable: the reference sources are not staged on this machine"
    print(json.dumps(out))
    return 0


def autograd_bench(args):
    """Differentiation workload: loss 0.5 ||FGP(f, lambda) - g||^2 over a batch of
    8 volumes of 128^3, 200 unrolled iterations, checkpoint every 20; forward and
    backward (hand-written adjoint) timed with CUDA events."""
    import torch
    from ccpi.filters.autograd import fgp_tv
    from ccpi.supp.phantoms import noisy_phantom

    f = torch.tensor(np.stack([noisy_phantom((128, 128, 128), 30, 4 + i) for i in range(8)]), device="cuda")
    g = torch.tensor(np.stack([noisy_phantom((128, 128, 128), 30, 400 + i) for i in range(8)]), device="cuda")
    iters, ckpt = 200, 20

    def step():
        fr = f.clone().requires_grad_(True)
        lam = torch.tensor(0.03, dtype=torch.float64, requires_grad=True)
        y = fgp_tv(fr, lam, iters, 0, 1, ckpt, batched=True)
        loss = 0.5 * ((y - g) ** 2).sum()
        loss.backward()
        return float(loss.detach()), float(lam.grad)

    step()
    times = []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        loss, lg = step()
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b) / 1e3)
    t = min(times)
    nvox = f.numel()
    print(json.dumps({"autograd": "FGP_TV 3D 8 x 128^3, 200 iterations, checkpoint 20, forward + adjoint",
                      "seconds_per_step": t, "volumes_per_s": 8 / t,
                      "forward_voxel_iters_per_s_equivalent": nvox * iters / t, "loss": loss, "dloss_dlambda": lg}))

    # the same for unrolled ROF-TV (lambda 0.02, tau 0.001)
    from ccpi.filters.autograd import rof_tv

    def rof_step():
        fr = f.clone().requires_grad_(True)
        lam = torch.tensor(0.02, dtype=torch.float64, requires_grad=True)
        y = rof_tv(fr, lam, iters, 0.001, ckpt, batched=True)
        loss = 0.5 * ((y - g) ** 2).sum()
        loss.backward()
        return float(loss.detach()), float(lam.grad)

    rof_step()
    times = []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        loss, lg = rof_step()
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b) / 1e3)
    t = min(times)
    print(json.dumps({"autograd": "ROF_TV 3D 8 x 128^3, 200 iterations, tau 0.001, checkpoint 20, forward + adjoint",
                      "seconds_per_step": t, "volumes_per_s": 8 / t,
                      "forward_voxel_iters_per_s_equivalent": nvox * iters / t, "loss": loss, "dloss_dlambda": lg}))
    return 0


def serve_requests(n, seed=3, rate=200.0):
    """The served workload: Poisson arrivals (mean `rate`/s), half 2D 1024^2,
    half 3D with edges from 128 to 384 (step 32); ROF / FGP / SB / NDF(Huber,
    sigma 0.02) uniformly; 5-50 outer FISTA steps of 20 inner iterations."""
    from ccpi.filters.serving import ProxRequest
    from ccpi.supp.phantoms import noisy_phantom

    rng = np.random.default_rng(seed)
    algs = [("ROF", (0.02, 0.001)), ("FGP", (0.03, 0, 1)), ("SB", (0.03, 0)), ("NDF", (0.02, 0.02, 0.01, 1))]
    cache = {}
    reqs, t = [], 0.0
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        if rng.random() < 0.5:
            shape = (1024, 1024)
        else:
            e = int(rng.choice(np.arange(128, 385, 32)))
            shape = (e, e, e)
        if shape not in cache:  # one phantom per size class, reused
            cache[shape] = noisy_phantom(shape, 30 if len(shape) == 3 else 10, 3)
        alg, prm = algs[int(rng.integers(0, 4))]
        reqs.append(ProxRequest(i, alg, cache[shape], prm, outer=int(rng.integers(5, 51)), inner=20, arrival=t))
    return reqs


def reference_fista(lib, req):
    """The plain per-call GPU path for one served request: FISTA on the host
    (numpy) around the reference's *_GPU_main called with host arrays for
    every prox (its state discarded after each call, TV_FGP_GPU_core.cu:586-598)."""
    f = np.ascontiguousarray(req.volume, dtype=np.float32)
    x, y, t = f.copy(), f.copy(), np.float32(1.0)
    st = np.float32(req.step)
    p = req.params
    for _ in range(req.outer):
        z = (y - st * (y - f)).astype(np.float32)
        if req.alg == "ROF":
            xn = _ref_call(lib, "TV_ROF_GPU_main", z, p[0], req.inner, p[1], 0.0)
        elif req.alg == "FGP":
            xn = _ref_call(lib, "TV_FGP_GPU_main", z, p[0], req.inner, 0.0, int(p[1]), int(p[2]))
        elif req.alg == "SB":
            xn = _ref_call(lib, "TV_SB_GPU_main", z, p[0], req.inner, 0.0, int(p[1]))
        else:
            xn = _ref_call(lib, "NonlDiff_GPU_main", z, p[0], p[1], req.inner, p[2], int(p[3]), 0.0)
        tn = np.float32((1.0 + np.sqrt(1.0 + 4.0 * t * t)) * 0.5)
        y = (xn + np.float32((t - 1.0) / tn) * (xn - x)).astype(np.float32)
        x, t = xn, tn
    return x


def serve_bench(args):
    """The served workload through the continuous-batching server, then the
    first --serve-ref-requests requests both through the server (all at once)
    and through the reference's plain per-call GPU path (one request after
    another, FISTA on the host, a cold reference prox per outer step)."""
    from ccpi.filters.serving import ProxServer, summarise

    reqs = serve_requests(args.requests)
    server = ProxServer(slots=8, hbm_budget=150e9)
    server.serve(reqs[:4], realtime=False)  # warm-up: module load, pool growth
    t = time.perf_counter()
    res = server.serve(reqs)
    wall = time.perf_counter() - t
    out = summarise(res, wall)
    out["workload"] = (f"{len(reqs)} prox requests, Poisson mean 200/s, 2D 1024^2 / 3D 128^3-384^3, "
                       "ROF/FGP/SB/NDF, 5-50 FISTA steps x 20 inner iterations, 8 slots, 150 GB budget")
    out["volumes_per_s"] = out["requests_per_s"]
    ref = reference_gpu_lib() if not args.no_reference_gpu else None
    if ref is not None:
        sub = reqs[:args.serve_ref_requests]
        reference_fista(ref, sub[0])  # module load, context
        t = time.perf_counter()
        for r in sub:
            reference_fista(ref, r)
        tr = time.perf_counter() - t
        t = time.perf_counter()
        mine = server.serve(sub, realtime=False)
        tm = time.perf_counter() - t
        assert all(m.ok for m in mine)
        out["reference_per_call"] = {
            "requests": len(sub), "voxel_iters": int(sum(r.volume.size * r.outer * r.inner for r in sub)),
            "reference_s": tr, "reference_requests_per_s": len(sub) / tr,
            "served_s": tm, "served_requests_per_s": len(sub) / tm, "speedup": tr / tm,
            "how": "the same requests, all available at once; reference: one request after another, FISTA on the "
                   "host around *_GPU_main with host arrays (cold prox state each outer step)"}
    else:
        out["reference_per_call"] = "unavailable: the reference sources are not staged on this machine"
    print(json.dumps({"serve": out}))
    return 0


def configs_bench(args):
    """Configs C1 (ROF 2D 512^2, 2000 iterations) and C2 (FGP and PD 3D at
    256^3 and 512^3, up to 500 iterations, epsil 1e-6) end to end through the
    reference-compatible Python API with host arrays (device='gpu'; copies
    included), each beside the reference CPU implementation on the host cores:
    C1 in full, C2 as a fixed 20-iteration sample (per-iteration cost is
    constant), projected to the iterations the GPU ran."""
    from ccpi.filters.regularisers import FGP_TV, PD_TV, ROF_TV
    from ccpi.supp.phantoms import noisy_phantom

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    use_ref = O.ref_lib() is not None
    kind, cores = ("reference" if use_ref else "port"), O.num_threads()

    def gpu_time(fn, reps=3):
        fn()
        ts = []
        for _ in range(reps):
            t = time.perf_counter()
            info = fn()
            ts.append(time.perf_counter() - t)
        return statistics.median(ts), info

    rows = []
    img = noisy_phantom((512, 512), 10, 0)

    def c1():
        info = np.zeros(2, np.float32)
        ROF_TV(img, 0.02, 2000, 0.001, 0.0, device="gpu", infovector=info)
        return info

    g, info = gpu_time(c1)
    t = time.perf_counter()
    O.rof_tv(img, 0.02, 2000, 0.001, 0.0, use_ref=use_ref)
    c = time.perf_counter() - t
    rows.append({"config": "C1 ROF_TV 2D 512^2, lambda 0.02, tau 0.001, 2000 iterations", "gpu_s": g,
                 "gpu_iterations": int(info[0]), "gpu_voxel_iters_per_s": img.size * 2000 / g, "cpu_s": c,
                 "cpu_sample": "full call", "cpu_kind": kind, "cpu_cores": cores, "speedup": c / g})
    for size in (256, 512):
        vol = noisy_phantom((size,) * 3, 30, 1)
        for name in ("FGP_TV", "PD_TV"):
            def call():
                info = np.zeros(2, np.float32)
                if name == "FGP_TV":
                    FGP_TV(vol, 0.03, 500, 1e-6, 0, 1, device="gpu", infovector=info)
                else:
                    PD_TV(vol, 0.03, 500, 1e-6, 8.0, 0, 1, device="gpu", infovector=info)
                return info

            g, info = gpu_time(call, reps=2)
            its = int(info[0])
            t = time.perf_counter()
            if name == "FGP_TV":
                O.fgp_tv(vol, 0.03, 20, 0.0, 0, 1, use_ref=use_ref)
            else:
                O.pd_tv(vol, 0.03, 20, 0.0, 8.0, 0, 1, use_ref=use_ref)
            c20 = time.perf_counter() - t
            cpu_rate = vol.size * 20 / c20
            c = vol.size * max(its, 1) / cpu_rate
            rows.append({"config": f"C2 {name} 3D {size}^3, lambda 0.03, up to 500 iterations, epsil 1e-6, iso, nonneg",
                         "gpu_s": g, "gpu_iterations": its, "gpu_voxel_iters_per_s": vol.size * its / g,
                         "cpu_s": c, "cpu_sample": f"20 fixed iterations ({c20:.1f} s), projected to {its}",
                         "cpu_kind": kind, "cpu_cores": cores, "cpu_voxel_iters_per_s": cpu_rate,
                         "speedup": c / g})
    for r in rows:
        print(json.dumps(r))
    print(json.dumps({"configs": rows}))
    return 0


def workload_figures():
    """Compact figures of the batched (64 uneven volumes, FGP and TGV, 300
    iterations, device-resident, one graph or persistent launch per
    regulariser as the autotuner picks) and served (48 prox requests, Poisson
    mean 200/s) workloads, added to the headline line so that every bench run
    records them.  The reference per-call legs of --batch / --serve take
    about a minute more and are left to those modes."""
    import torch
    from ccpi.filters.batch import FGP_TV_batch, TGV_batch
    from ccpi.filters.serving import ProxServer, summarise

    vols = [torch.from_numpy(v).cuda() for v in batch_volumes()]
    nvox = sum(v.numel() for v in vols)
    out = {}
    for name, fn in (("FGP_TV", lambda: FGP_TV_batch(vols, 0.03, 300, 0.0, 0, 1)),
                     ("TGV", lambda: TGV_batch(vols, 0.03, 1.0, 2.0, 300, 12.0))):
        fn()  # warm-up (the autotuner times its candidates on the first call of a layout)
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        out[name] = {"seconds": dt, "volumes_per_s": len(vols) / dt, "voxel_iters_per_s": nvox * 300 / dt}
    batched = {"workload": f"{len(vols)} volumes, edges from {{96,...,256}}, {nvox} voxels, 300 iterations",
               **out}
    del vols
    reqs = serve_requests(48)
    server = ProxServer(slots=8, hbm_budget=150e9)
    server.serve(reqs[:4], realtime=False)
    t = time.perf_counter()
    res = server.serve(reqs)
    served = summarise(res, time.perf_counter() - t)
    served["workload"] = "48 prox requests, Poisson mean 200/s, 2D 1024^2 / 3D 128^3-384^3, 5-50 FISTA x 20"
    return {"batched": batched, "served": served}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--ref-iters", type=int, default=20, help="iterations per reference-arm step")
    ap.add_argument("--cpu-iters", type=int, default=20, help="iterations of the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-workloads", action="store_true",
                    help="leave the batched and served figures out of the headline line")
    ap.add_argument("--profile-case", action="store_true",
                    help="only run --steps FGP calls of --iters fixed iterations on the device (for ncu)")
    ap.add_argument("--iters", type=int, default=20, help="iterations per call in --profile-case")
    ap.add_argument("--reg", default="FGP",
                    help="regulariser of --profile-case (FGP, ROF, PD, SB, TGV, NDF, Diff4th, LLT_ROF, FGP_dTV)")
    ap.add_argument("--batch", action="store_true",
                    help="64 uneven volumes, FGP and TGV at 300 iterations: batched graph launch vs per-call")
    ap.add_argument("--autograd", action="store_true",
                    help="unrolled FGP-TV forward + adjoint on 8 volumes of 128^3, 200 iterations, checkpoint 20")
    ap.add_argument("--serve", action="store_true",
                    help="Poisson stream (mean 200 req/s) of prox requests through the continuous-batching server")
    ap.add_argument("--requests", type=int, default=48, help="requests of the --serve stream")
    ap.add_argument("--serve-ref-requests", type=int, default=12,
                    help="requests of the --serve stream also run through the reference's per-call GPU path")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="--batch / --serve: skip the reference's per-call GPU path")
    ap.add_argument("--configs", action="store_true",
                    help="configs C1 and C2 through the Python API (host arrays) beside the reference CPU")
    ap.add_argument("--regs", default="", help="comma-separated regularisers of --suite (default: all)")
    ap.add_argument("--suite", action="store_true",
                    help="per-regulariser iteration time and roofline fraction (device data, fixed counts)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_case:
        return profile_case(args)
    if args.suite:
        return suite(args)
    if args.configs:
        return configs_bench(args)
    if args.batch:
        return batch_bench(args)
    if args.autograd:
        return autograd_bench(args)
    if args.serve:
        return serve_bench(args)

    import ctypes

    import torch

    rank, world, local = _env_rank()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
        pg = dist

    from ccpi.filters import utils as U

    lib = U.cilregcuda
    x = _phantom(args.size)
    n = x.size
    nx = ny = nz = args.size
    stream = torch.cuda.current_stream(dev)
    d_in = torch.from_numpy(x).to(dev)
    d_out = torch.zeros_like(d_in)
    info = np.zeros(2, np.float32)
    info_p = info.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    def step(iters=MAX_ITERS, epsil=EPSIL):
        d_out.zero_()  # U_prev of iteration 0, as the reference's np.zeros_like output
        st = lib.cilreg_fgp_tv_dev(d_in.data_ptr(), d_out.data_ptr(), info_p, LAM, iters, epsil, METHOD, NONNEG,
                                   nx, ny, nz, stream.cuda_stream)
        U.check_status(st)
        return int(info[0])

    for _ in range(args.warmup):
        step()

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize(dev)

    clocks = ClockSampler(local)
    clocks.start()
    launches0 = U.launch_count()
    barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    iters_run = 0
    ev0.record(stream)
    for _ in range(args.steps):
        iters_run += step()
    ev1.record(stream)
    barrier()
    launches = U.launch_count() - launches0
    clock_info = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    t_local = ms / 1e3
    t_max, total_vi = reduce_over_ranks(pg, t_local, n * iters_run, dev)
    value = total_vi / t_max

    # steady-state launch time of the FGP iteration kernel: difference of two
    # fixed-count runs on the same stream (one kernel launch per iteration)
    def timed(iters):
        barrier()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step(iters, 0.0)
        b.record(stream)
        torch.cuda.synchronize(dev)
        return a.elapsed_time(b) / 1e3

    i1, i2 = 10, 60
    timed(i1)
    t1 = min(timed(i1) for _ in range(2))
    t2 = min(timed(i2) for _ in range(2))
    per_launch = (t2 - t1) / (i2 - i1)
    peak, peak_kind = _peaks()
    achieved = BYTES_PER_VOXEL_ITER * n / per_launch / 1e9
    tpv = _ncu_traffic_per_voxel()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": (tpv * n if tpv is not None else None), "peak_kind": peak_kind,
                "traffic_source": ("not measured in this run: the ncu DRAM bytes per voxel-iteration of "
                                   "profiles/fgp_tv_3d_kernel.md scaled to this launch"),
                "kernel": fgp_kernel_name(nx), "launch_ms": per_launch * 1e3,
                "algorithmic_bytes_per_launch": BYTES_PER_VOXEL_ITER * n}

    # end to end through the reference-facing C ABI with pinned host buffers
    h_in = torch.from_numpy(x).pin_memory()
    h_out = torch.zeros_like(h_in).pin_memory()
    fp = ctypes.POINTER(ctypes.c_float)
    e2e_steps = max(1, min(args.steps, 3))
    lib.TV_FGP_GPU_main(ctypes.cast(h_in.data_ptr(), fp), ctypes.cast(h_out.data_ptr(), fp), info_p, LAM, MAX_ITERS,
                        EPSIL, METHOD, NONNEG, local, nx, ny, nz)
    # the GPU entry point never reads Output (it is written whole), so the
    # buffer is cleared once, outside the timed region, and checked after it
    h_out.zero_()
    # this machine's host <-> device copy rate (pinned, one 4 n-byte copy each
    # way), reported beside e2e: the copies are e2e's only extra work
    d_tmp = torch.empty_like(h_in, device=dev)
    copy_gbs = {}
    for name, dst, src in (("h2d", d_tmp, h_in), ("d2h", h_out, d_tmp)):
        best = None
        for _ in range(3):
            torch.cuda.synchronize(dev)
            tc = time.perf_counter()
            dst.copy_(src, non_blocking=True)
            torch.cuda.synchronize(dev)
            tc = time.perf_counter() - tc
            best = tc if best is None else min(best, tc)
        copy_gbs[name] = 4 * n / best / 1e9
    del d_tmp
    h_out.zero_()
    barrier()
    e2e_vi = 0
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        st = lib.TV_FGP_GPU_main(ctypes.cast(h_in.data_ptr(), fp), ctypes.cast(h_out.data_ptr(), fp), info_p, LAM,
                                 MAX_ITERS, EPSIL, METHOD, NONNEG, local, nx, ny, nz)
        U.check_status(st)
        e2e_vi += n * int(info[0])
    barrier()
    e2e_t = time.perf_counter() - t0
    if not bool(torch.isfinite(h_out).all()) or float(h_out.abs().max()) == 0.0:
        raise RuntimeError("the end-to-end call left Output empty or non-finite")
    e2e_t_max, e2e_vi_all = reduce_over_ranks(pg, e2e_t, e2e_vi, dev)
    e2e_val = e2e_vi_all / e2e_t_max

    # the same through the reference-facing Python call with pageable numpy
    # arrays, as the reference's callers make it (TV.py:524-565): a fresh
    # output array per call, infovector returned, copies inside the call
    from ccpi.filters.regularisers import FGP_TV

    info_py = np.zeros(2, np.float32)
    FGP_TV(x, LAM, MAX_ITERS, EPSIL, METHOD, NONNEG, device="gpu", infovector=info_py)
    barrier()
    py_vi, py_times = 0, []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        out_py = FGP_TV(x, LAM, MAX_ITERS, EPSIL, METHOD, NONNEG, device="gpu", infovector=info_py)
        py_times.append(time.perf_counter() - t0)
        py_vi += n * int(info_py[0])
    barrier()
    if not bool(np.isfinite(out_py).all()) or float(np.abs(out_py).max()) == 0.0:
        raise RuntimeError("the Python-API call left its output empty or non-finite")
    py_t_max, py_vi_all = reduce_over_ranks(pg, sum(py_times), py_vi, dev)

    workloads = None
    if rank == 0 and world == 1 and not args.no_workloads:
        workloads = workload_figures()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, kind, cores, dt = cpu_baseline(x, args.cpu_iters)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": kind,
               "sample": f"FGP_TV {args.size}^3, {args.cpu_iters} fixed iterations (epsil=0), {dt:.1f} s",
               **host_info()}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"FGP_TV 3D {args.size}^3 ellipsoid phantom + noise", "lambda": LAM,
                       "max_iterations": MAX_ITERS, "epsil": EPSIL, "methodTV": "iso", "nonneg": NONNEG,
                       "iterations_per_step": iters_run / args.steps,
                       "l2": "inputs larger than L2 (state 5.6 GB per replica, L2 126 MB)",
                       "parallelism": f"replicas x{world}"},
            "roofline": roofline,
            "cpu_baseline": cpu,
            # the input goes up, the result comes back (U_prev of iteration 0 is zeroed on the device)
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": 4 * n,
                    "copy_gbs": copy_gbs},
            "e2e_python_api": {"value": py_vi_all / py_t_max, "unit": UNIT, "h2d_bytes_per_step": 4 * n,
                               "d2h_bytes_per_step": 4 * n, "ms_per_call": [1e3 * t for t in py_times],
                               "how": "ccpi.filters.regularisers.FGP_TV(numpy array, device='gpu'): pageable "
                                      "host arrays, a new output array per call"},
            "gpu_launches": launches,
            "clocks": clock_info,
            "workloads": workloads,
        }
        print(json.dumps(line))
    if pg is not None:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
