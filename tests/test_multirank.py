"""The multi-process (replicas) logic of bench.py on CPU ranks with gloo:
each rank runs its own copy of the workload; the whole-job figure is the sum of
all ranks' voxel-iterations over the slowest rank's time, and the reference
arm runs on rank 0 only."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r took (1 + r) s for 100 (r + 1) voxel-iterations
    t, units = bench.reduce_over_ranks(dist, 1.0 + rank, 100.0 * (rank + 1), torch.device("cpu"))
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out, f"rank{rank}.json"), "w") as f:
        json.dump({"t": t, "units": units}, f)


@pytest.mark.parametrize("world", [2, 3])
def test_replica_figures_reduce_over_gloo_ranks(world, tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.spawn(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    want_t = float(world)
    want_units = 100.0 * world * (world + 1) / 2
    for r in range(world):
        got = json.loads((tmp_path / f"rank{r}.json").read_text())
        assert got["t"] == want_t
        assert got["units"] == want_units


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_over_ranks(None, 2.5, 7, None) == (2.5, 7.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        size, ref_iters, warmup, steps, gpus = 512, 4, 3, 2, 2

    assert bench.run_reference(Args()) == 0
    assert capsys.readouterr().out == ""
