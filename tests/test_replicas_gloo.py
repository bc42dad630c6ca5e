"""The multi-GPU path is replicas only: each rank advances its own copy and the
job's time is the slowest rank's.  Its host logic (process group set-up,
max-reduce of the timing, the whole-job rate) runs here as two gloo ranks on
the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank), "CUDA_VISIBLE_DEVICES": ""})
    import bench

    dist, r, w, _ = bench.dist_setup(world)
    assert (r, w) == (rank, world) and dist.get_backend() == "gloo"
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist)
    out[rank] = (ms, bench.job_rate(w, 1000, 4, ms))
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world = 2
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    ms, rate = res[0]
    assert ms == 15.0
    assert rate == pytest.approx(2 * 1000 * 4 / 15e-3)
