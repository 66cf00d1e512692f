"""Id-range sharding: every rank holds the objects [offset, offset + n) of the
table under local ids and answers the same queries; one exchange gathers the
per-rank top-k lists and merges them into the global top-k (exact: counts are
per object).  No collective runs inside the search itself."""
import ctypes

import numpy as np


def shard_range(n_objects, rank, world):
    """[a, b) of the objects that rank holds."""
    return n_objects * rank // world, n_objects * (rank + 1) // world


def merge(results, offsets, k, scores=None):
    """Global top-k from per-shard (ids, counts) lists of the same queries.
    results: [(ids, counts), ...]; offsets: first global id of each shard;
    k: scalar or one value per query.  scores: per-shard score arrays or None."""
    from . import _check, lib
    n = len(results)
    ids = [np.ascontiguousarray(r[0], np.uint32) for r in results]
    cnt = [np.ascontiguousarray(r[1], np.uint32) for r in results]
    sc = None if scores is None else [np.ascontiguousarray(s, np.float32) for s in scores]
    total = len(ids[0])
    if np.isscalar(k):
        kk, uk, nq = None, int(k), total // int(k)
    else:
        kk = np.ascontiguousarray(k, np.uint32)
        uk, nq = 0, len(kk)
    P = ctypes.c_void_p * n
    out_ids = np.zeros(max(1, total), np.uint32)
    out_cnt = np.zeros(max(1, total), np.uint32)
    out_sc = np.zeros(max(1, total), np.float32) if sc is not None else None
    off = np.ascontiguousarray(offsets, np.int64)
    _check(lib().genie_merge_shards(n, P(*[a.ctypes.data for a in ids]), P(*[a.ctypes.data for a in cnt]),
                                    None if sc is None else P(*[a.ctypes.data for a in sc]), off.ctypes.data,
                                    nq, None if kk is None else kk.ctypes.data, uk, out_ids.ctypes.data,
                                    out_cnt.ctypes.data, None if out_sc is None else out_sc.ctypes.data))
    if out_sc is None:
        return out_ids[:total], out_cnt[:total]
    return out_ids[:total], out_cnt[:total], out_sc[:total]


def gather_merge(ids, counts, offset, k, group=None, scores=None):
    """torch.distributed exchange: every rank passes its shard's results of the
    same queries; rank 0 gets the merged global top-k, the others None."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    cols = [np.asarray(ids, np.int64), np.asarray(counts, np.int64)]
    if scores is not None:
        cols.append(np.asarray(scores, np.float32).view(np.int32).astype(np.int64))
    mine = torch.from_numpy(np.stack(cols + [np.full(len(cols[0]), offset, np.int64)]))
    if dist.get_backend(group) == "nccl":
        mine = mine.cuda()
    parts = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine, group=group)
    if rank != 0:
        return None
    parts = [p.cpu().numpy() for p in parts]
    res = [(p[0], p[1]) for p in parts]
    offs = [int(p[-1][0]) if p.shape[1] else 0 for p in parts]
    sc = None if scores is None else [p[2].astype(np.int32).view(np.float32) for p in parts]
    return merge(res, offs, k, sc)
