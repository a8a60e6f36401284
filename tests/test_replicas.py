"""The N>1 path of bench.py on CPU: two gloo ranks, each timing its own
replica, agree on the slowest rank's time and on the whole-job rate."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from godunov_five_eq_gb300.replicas import max_over_ranks, rank_env, whole_job_rate  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, local = rank_env()
    assert (w, r, local) == (world, rank, rank)
    my_ms = 10.0 + 5.0 * rank  # the replicas' own timings differ
    dist.barrier()
    slowest = max_over_ranks(my_ms)
    rate = whole_job_rate(w, 431104, 20, slowest)
    out[rank] = (slowest, rate)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_agree():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    slowest, rate = res[0]
    assert slowest == 15.0
    assert rate == pytest.approx(2 * 431104 * 20 / 15e-3)


def test_single_process_defaults():
    assert max_over_ranks(3.5) == 3.5
    assert whole_job_rate(1, 100, 10, 1000.0) == pytest.approx(1000.0)
