"""bench.py's multi-GPU logic on CPU: replicas only, so the one cross-rank
exchange is the timing (a barrier and a max over ranks).  Two gloo ranks on
127.0.0.1 check it; the CPU reference arm runs on rank 0 only."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    ms = bench.reduce_max(100.0 + 50.0 * rank, world)
    value = bench.aggregate_value(world, 256 ** 3, 5, ms)
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_max_timing_and_aggregate():
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
    assert out[0][0] == out[1][0] == 150.0
    assert out[0][1] == out[1][1] == 2 * 256 ** 3 * 5 / 0.150


def test_reference_arm_runs_on_rank_zero_only(capsys):
    import bench

    class A:
        N = 8
        steps = 1
        warmup = 0
        gpus = 2

    bench.run_reference(A, rank=1, world=2)
    assert capsys.readouterr().out == ""
