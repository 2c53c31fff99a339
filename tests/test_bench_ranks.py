"""The N-replica path of bench.py on CPU: rank environment parsing and the max-over-ranks
timing, run as two gloo ranks (the GPU bench uses the same functions over NCCL)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as tdist

    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    r, w, local = bench.dist_env()
    assert (r, w, local) == (rank, world, rank)
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.replica_time_ms(100.0 + 50.0 * rank, world, "cpu")
        tdist.barrier()
        out[rank] = (ms, bench.aggregate_rate(200, ms, world))
    finally:
        tdist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    assert out[0] == out[1]
    ms, rate = out[0]
    assert ms == pytest.approx(150.0)
    assert rate == pytest.approx(2 * 200 / 0.150)


def test_single_rank_defaults(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_env() == (0, 1, 0)
    assert bench.replica_time_ms(12.5, 1, "cpu") == 12.5
