"""CPU checks of the ensemble host logic: instance set-up and the sharding of instances across
ranks (world size 2 over gloo; no data-path exchange, the ranks only compare their shares)."""
import os

import numpy as np
import pytest


def test_instances_follow_their_seeds():
    from festung_gb300 import ensemble as E
    from festung_gb300 import testcases as TC
    for seed in (0, 5):
        pd = E.instance_problem(seed, numSteps=4, setupOnDevice=False)
        prm = TC.ensemble_params(seed)
        assert pd.p == prm['p'] and pd.hmax == prm['hmax']
        assert pd.K % 128 == 0 and pd.K in (2048, 8192, 32768)
        assert pd.c0.shape == (pd.K, pd.N) and pd.u1Disc.shape == (pd.K, pd.N)
        dev = E.instance_problem(seed, numSteps=4)
        assert dev.deviceFns['c0'][1][2] == prm['width'] ** 2 and 'u1Disc' not in dev


def test_shard_partitions_instances():
    from festung_gb300 import ensemble as E
    for n in (1, 7, 256):
        for world in (1, 2, 3, 8):
            parts = [E.shard(n, r, world) for r in range(world)]
            flat = sorted(i for p in parts for i in p)
            assert flat == list(range(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1


def _rank(rank, world, port, n, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    from festung_gb300 import ensemble as E
    mine = E.shard(n, rank, world)
    out = [None] * world
    dist.all_gather_object(out, mine)
    dist.destroy_process_group()
    q.put((rank, out))


def test_two_ranks_share_out_the_instances():
    import multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, 256, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    for rank, out in res:
        assert sorted(out[0] + out[1]) == list(range(256))
        assert not set(out[0]) & set(out[1])
