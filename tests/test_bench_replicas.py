"""Host logic of the multi-rank bench (replicas only): two gloo ranks on the
CPU combine their lines into the whole-job line -- the slowest rank's time,
the cell updates of all ranks."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _line(ms, e2e):
    return {"ms_per_step": ms, "value": 1e6 / (ms * 1e-3), "n_gpus": 1, "gpu_launches": 70,
            "config": {"cells": 1_000_000}, "e2e": {"value": e2e, "unit": "cell-updates/s"}}


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch

    def allreduce_max(vals):
        t = torch.tensor(vals, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return t.tolist()

    dist.barrier()
    # rank 1 is the slow one in the device-timed run, rank 0 in the e2e run
    line = _line(ms=2.0 if rank == 1 else 1.0, e2e=1e8 if rank == 0 else 3e8)
    q.put((rank, bench.combine_replicas(line, world, allreduce_max)))
    dist.destroy_process_group()


def test_combine_replicas_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        out = got[r]
        assert out["ms_per_step"] == 2.0  # the slowest rank
        assert out["value"] == pytest.approx(2 * 1_000_000 / 2e-3)
        assert out["e2e"]["value"] == pytest.approx(2 * 1e8)
        assert out["n_gpus"] == 2 and out["gpu_launches"] == 140


def test_launches_per_step():
    from rift_gb300 import synth
    assert bench.launches_per_step(synth.RAIN_UNIFORM) == 7
    assert bench.launches_per_step(synth.RAIN_GRID) == 8
    assert bench.launches_per_step(synth.EULER | synth.SURGE_GRID) == 7
