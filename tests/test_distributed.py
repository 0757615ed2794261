"""Multi-rank host logic on CPU with gloo (world size 2): replica timing aggregation, ensemble
slicing, and detection of a rank that fails before the aggregation."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from phasefield_gb300 import replicas


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, results, fail_rank):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import datetime
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    try:
        if rank == fail_rank:
            raise RuntimeError("planted failure")
        ms, work = replicas.aggregate(10.0 + rank, 1000 * (rank + 1), dist)
        results[rank] = (ms, work)
    except RuntimeError as e:
        results[rank] = ("error", str(e))
    finally:
        dist.destroy_process_group()


def _run(world, fail_rank=-1):
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        results = m.dict()
        mp.spawn(_worker, args=(world, port, results, fail_rank), nprocs=world, join=True)
        return dict(results)


def test_aggregate_max_time_sum_work_world2():
    res = _run(2)
    assert res[0] == (11.0, 3000)
    assert res[1] == (11.0, 3000)


def test_failed_rank_is_reported_not_hung():
    # rank 1 raises before the collective; rank 0's collective ends with an error after the
    # process-group timeout instead of hanging
    res = _run(2, fail_rank=1)
    assert res[1][0] == "error"
    assert res[0][0] == "error"


def test_split_instances_covers_all_once():
    for n in (1, 7, 256):
        for world in (1, 2, 3, 8):
            seen = [i for r in range(world) for i in replicas.split_instances(n, r, world)]
            assert seen == list(range(n))


def test_single_process_aggregate_is_identity():
    assert replicas.aggregate(5.0, 42) == (5.0, 42)
