"""Multi-rank bookkeeping on CPU: two gloo ranks, as bench.py --gpus 2 uses it."""
import os

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from ugacc_gb300.replicas import allmax, shard, whole_job_rate


def test_shard_covers_all_items_once():
    for n in (0, 1, 7, 512):
        for w in (1, 2, 3, 8):
            got = [i for r in range(w) for i in shard(n, r, w)]
            assert got == list(range(n))
            sizes = [len(shard(n, r, w)) for r in range(w)]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [3.0, 5.0][rank]
        t, value = whole_job_rate(100.0, ms, world, dist)
        out[rank] = (allmax(float(rank), dist), t, value)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_max_time_and_rate():
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for r in (0, 1):
        mx, t, value = res[r]
        assert mx == 1.0 and t == 5.0
        assert value == pytest.approx(2 * 100.0 / 5.0)
