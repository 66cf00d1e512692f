"""Id-range sharding: the per-shard top-k lists of the same
queries merge into the global top-k.  The merge is host code; the exchange is
a torch.distributed all_gather, run here as two gloo ranks on the CPU.  The
per-shard searches in these tests are the oracle's (the GPU path per shard is
genie_search on the shard's table, tested elsewhere)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _shard_results(values, batch, a, b):
    from oracle import oracle
    sub = oracle.Index(values[a:b])
    ids, cnt, sc, _ = sub.search(batch)
    return ids, cnt, sc


def _genie():
    from genie_gb300 import build
    build.build()
    import genie_gb300
    return genie_gb300


def test_merge_equals_unsharded_top_k(oracle):
    genie = _genie()
    from genie_gb300 import workloads
    values, batch = workloads.config3(n=30_000, q=40)
    batch = dict(batch)
    full_ids, full_cnt, full_sc, _ = oracle.Index(values).search(batch)
    for world in (2, 3):
        res, scs, offs = [], [], []
        for r in range(world):
            a, b = genie.shard.shard_range(len(values), r, world)
            ids, cnt, sc = _shard_results(values, batch, a, b)
            res.append((ids, cnt))
            scs.append(sc)
            offs.append(a)
        ids, cnt, sc = genie.shard.merge(res, offs, batch["k"], scores=scs)
        unweighted = np.repeat(batch["weighted"] == 0, batch["k"])
        # unweighted queries: exact
        assert np.array_equal(ids[unweighted], full_ids[unweighted])
        assert np.array_equal(cnt[unweighted], full_cnt[unweighted])
        # weighted queries: same score multiset (ids may swap only between equal float scores)
        assert np.array_equal(sc[~unweighted], full_sc[~unweighted])


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from genie_gb300 import workloads
    import genie_gb300 as genie
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    values, batch = workloads.config1(n=20_000, q=24, k=10)
    a, b = genie.shard.shard_range(len(values), rank, world)
    ids, cnt, _ = _shard_results(values, batch, a, b)
    merged = genie.shard.gather_merge(ids, cnt, a, 10)
    if rank == 0:
        np.save(os.path.join(out_dir, "ids.npy"), merged[0])
        np.save(os.path.join(out_dir, "cnt.npy"), merged[1])
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_and_merge(oracle, tmp_path):
    _genie()
    import torch.multiprocessing as mp
    from genie_gb300 import workloads
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    values, batch = workloads.config1(n=20_000, q=24, k=10)
    oid, ocnt, _, _ = oracle.Index(values).search(batch)
    assert np.array_equal(np.load(tmp_path / "ids.npy"), oid)
    assert np.array_equal(np.load(tmp_path / "cnt.npy"), ocnt)
