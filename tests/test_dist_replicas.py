"""The multi-GPU path is replicas only: every rank runs the whole workload on its own GPU
and bench.py reports the whole job -- all ranks' units over the slowest rank's time
(job_rate, a max all-reduce).  Checked here with two gloo ranks on the CPU (127.0.0.1), and
the reference arm's rule that only rank 0 times and prints."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [40.0, 55.0][rank]
    value, slowest = bench.job_rate(dist, ms, world, 1000.0, device="cpu")
    out[rank] = (value, slowest)
    dist.destroy_process_group()


def test_job_rate_is_all_units_over_the_slowest_rank():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        value, slowest = res[r]
        assert slowest == 55.0
        assert value == pytest.approx(2 * 1000.0 / 0.055)


def test_reference_arm_prints_on_rank_zero_only(capsys, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        steps, warmup, gpus = 1, 1, 2
    assert bench.run_reference(Args()) == 0
    assert capsys.readouterr().out == ""
