"""Multi-rank host logic on CPU: two gloo ranks split a request list by key,
each signs its share with the oracle (standing in for its GPU), and the
gathered results equal one rank signing everything."""
import os
import random
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _requests():
    rng = random.Random(8)
    keys = [bytes(rng.randrange(256) for _ in range(48)) for _ in range(5)]
    reqs = [(rng.randrange(5), bytes(rng.randrange(256) for _ in range(rng.randrange(0, 80)))) for _ in range(10)]
    return keys, reqs


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    import spx_oracle
    from cuspx_gb300 import replicas
    o = spx_oracle.Oracle("sha256-128f-simple")
    keys, reqs = _requests()
    sks = [o.seed_keypair(k)[1] for k in keys]
    mine = replicas.shard_by_key([k for k, _ in reqs], rank, world)
    part = [(i, o.sign(reqs[i][1], sks[reqs[i][0]]).hex()) for i in mine]
    gathered = [None] * world
    dist.all_gather_object(gathered, part)
    if rank == 0:
        out.put(replicas.merge(gathered, len(reqs)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_by_key():
    torch = pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import spx_oracle
    o = spx_oracle.Oracle("sha256-128f-simple")
    keys, reqs = _requests()
    sks = [o.seed_keypair(k)[1] for k in keys]
    assert merged == [o.sign(m, sks[k]).hex() for k, m in reqs]


def test_merge_rejects_gaps_and_duplicates():
    from cuspx_gb300 import replicas
    with pytest.raises(ValueError):
        replicas.merge([[(0, "a")], [(0, "b")]], 1)
    with pytest.raises(ValueError):
        replicas.merge([[(0, "a")], []], 2)
    assert replicas.shard_by_key([0, 1, 2, 3, 4], 1, 2) == [1, 3]
