"""Batched search (CUDA graph, device-side batch size, autotuner) against
the oracle and the plain per-batch path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _qb(genie, b):
    return genie.QueryBatch(b["item_off"], b["dim"], b["low"], b["up"], b["k"], b.get("weight"), b.get("weighted"))


def _slice(b, q0, q1):
    off = b["item_off"]
    a, z = off[q0], off[q1]
    out = dict(item_off=off[q0:q1 + 1] - a, dim=b["dim"][a:z], low=b["low"][a:z], up=b["up"][a:z],
               k=b["k"][q0:q1])
    if b.get("weight") is not None:
        out["weight"] = b["weight"][a:z]
        out["weighted"] = b["weighted"][q0:q1]
    return out


def test_graph_batch_varying_sizes(genie, oracle):
    from genie_gb300 import workloads
    values, batch = workloads.config3(n=300_000, q=64)
    t = genie.Table.from_values(values)
    ox = oracle.Index(values)
    bt = genie.Batch(t, max_queries=64, max_items=int(batch["item_off"][-1]), max_k=100)
    for q0, q1 in ((0, 64), (5, 9), (10, 60), (0, 1)):
        sub = _slice(batch, q0, q1)
        qb = _qb(genie, sub)
        ids, cnt, sc = bt.run(qb, scores=True)
        oid, ocnt, osc, _ = ox.search(qb.as_oracle_batch())
        assert np.array_equal(ids, oid) and np.array_equal(cnt, ocnt) and np.array_equal(sc, osc)
        pid, pcnt = genie.search(t, qb)
        assert np.array_equal(ids, pid) and np.array_equal(cnt, pcnt)
    kernels, ms = bt.last_stats()
    assert kernels >= 4 and ms > 0      # the plan, the bitmap, sparse and dense kernels


def test_stage_launch_fetch_repeatable(genie, oracle):
    from genie_gb300 import workloads
    values, batch = workloads.config1(n=100_000, q=64, k=100)
    t = genie.Table.from_values(values)
    qb = _qb(genie, batch)
    bt = genie.Batch(t, 64, int(batch["item_off"][-1]), 100)
    bt.stage(qb)
    first = None
    for _ in range(3):
        bt.launch()
        got = bt.fetch()
        if first is None:
            first = got
        assert all(np.array_equal(a, b) for a, b in zip(got, first))
    oid, ocnt, _, _ = oracle.Index(values).search(qb.as_oracle_batch())
    assert np.array_equal(first[0], oid) and np.array_equal(first[1], ocnt)


def test_autotune_keeps_results_exact(genie, oracle):
    from genie_gb300 import workloads
    values, batch = workloads.config3(n=200_000, q=32)
    t = genie.Table.from_values(values)
    qb = _qb(genie, batch)
    bt = genie.Batch(t, 32, int(batch["item_off"][-1]), 100)
    chosen = bt.autotune(qb)
    assert chosen["sparse_slots"] > 0 and chosen["dense_tile"] > 0
    ids, cnt = bt.run(qb)
    oid, ocnt, _, _ = oracle.Index(values).search(qb.as_oracle_batch())
    assert np.array_equal(ids, oid) and np.array_equal(cnt, ocnt)
    # a smaller hash (more parts per query) and a smaller tile give the same answer
    bt.set_tuning(sparse_slots=4096, dense_tile=16384)
    ids2, cnt2 = bt.run(qb)
    assert np.array_equal(ids2, oid) and np.array_equal(cnt2, ocnt)
    # one 1024-thread CTA per SM with the largest table and a higher load
    bt.set_tuning(sparse_slots=53248, sparse_ctas_per_sm=1, sparse_load_pct=62, dense_tile=147456)
    ids3, cnt3 = bt.run(qb)
    assert np.array_equal(ids3, oid) and np.array_equal(cnt3, ocnt)
    with pytest.raises(genie.cpu_runtime_error):
        bt.set_tuning(sparse_load_pct=95)


def test_big_table_variant_on_lsh_batch(genie, oracle):
    from genie_gb300 import workloads
    values, batch = workloads.config1(n=300_000, q=48, k=100)
    t = genie.Table.from_values(values)
    qb = _qb(genie, batch)
    bt = genie.Batch(t, 48, int(batch["item_off"][-1]), 100)
    bt.set_tuning(sparse_slots=53248, sparse_ctas_per_sm=1, sparse_load_pct=62)
    ids, cnt = bt.run(qb)
    oid, ocnt, _, _ = oracle.Index(values).search(qb.as_oracle_batch())
    assert np.array_equal(ids, oid) and np.array_equal(cnt, ocnt)


@pytest.mark.parametrize("n", [100_000, 300_000, 1_000_000])
def test_bitmap_kernel_modes(genie, oracle, n):
    """The presence-bitmap kernel (the table of repeated ids holding fewer or
    more than k ids), the hash kernel when the id space exceeds the bitmap
    limit, and the bitmap kernel switched off give the oracle's answer."""
    from genie_gb300 import workloads
    values, batch = workloads.config1(n=n, q=32, k=100)
    t = genie.Table.from_values(values)
    qb = _qb(genie, batch)
    oid, ocnt, _, _ = oracle.Index(values).search(qb.as_oracle_batch())
    bt = genie.Batch(t, 32, int(batch["item_off"][-1]), 100)
    for bits in (1179648, 8192, -1):
        bt.set_tuning(bitmap_bits=bits)
        assert bt.tuning()["bitmap_bits"] == bits
        ids, cnt = bt.run(qb)
        assert np.array_equal(ids, oid) and np.array_equal(cnt, ocnt), bits


def test_bitmap_overflow_retries_dense(genie, oracle):
    """Queries whose repeated ids overflow the bitmap kernel's table are redone
    by the dense kernel with the same answer."""
    rng = np.random.default_rng(7)
    values = rng.integers(0, 4, size=(200_000, 16), dtype=np.int32)
    q, m = 8, 3
    dims = np.tile(np.arange(m, dtype=np.int32), q)
    vals = rng.integers(0, 4, size=q * m).astype(np.int32)
    qb = genie.QueryBatch(np.arange(q + 1) * m, dims, vals, vals, 50)
    t = genie.Table.from_values(values)
    bt = genie.Batch(t, q, q * m, 50, use_graph=False)
    bt.set_tuning(sparse_max_total=1081344, bitmap_bits=1310720)
    ids, cnt = bt.run(qb)
    ms = bt.stage_ms()
    assert ms.shape == (4,) and ms[1] > 0
    oid, ocnt, _, _ = oracle.Index(values).search(qb.as_oracle_batch())
    assert np.array_equal(ids, oid) and np.array_equal(cnt, ocnt)


def test_bitmap_ties_in_one_id_range(genie, oracle):
    """Many ids tied at the k-th count inside one small id range (identical
    objects with adjacent ids) are still returned in ascending id order."""
    rng = np.random.default_rng(11)
    values = rng.integers(0, 1000, size=(100_000, 16), dtype=np.int32)
    values[:40] = values[0]
    q = 6
    dims = np.tile(np.arange(16, dtype=np.int32), q)
    vals = rng.integers(0, 1000, size=(q, 16)).astype(np.int32)
    vals[:, :5] = values[0, :5]
    vals = vals.ravel()
    qb = genie.QueryBatch(np.arange(q + 1) * 16, dims, vals, vals, 10)
    t = genie.Table.from_values(values)
    bt = genie.Batch(t, q, q * 16, 10)
    ids, cnt = bt.run(qb)
    oid, ocnt, _, _ = oracle.Index(values).search(qb.as_oracle_batch())
    assert np.array_equal(ids, oid) and np.array_equal(cnt, ocnt)
    assert list(ids[:10]) == list(range(10))


def test_batch_capacity_errors(genie):
    t = genie.Table.from_values(np.zeros((10, 2), np.int32))
    bt = genie.Batch(t, 2, 4, 5)
    with pytest.raises(genie.cpu_runtime_error):
        bt.run(genie.QueryBatch([0, 1, 2, 3], [0, 0, 0], [0, 0, 0], [0, 0, 0], 5))
    with pytest.raises(genie.cpu_runtime_error):
        bt.run(genie.QueryBatch([0, 1], [0], [0], [0], 6))
    ids, cnt = bt.run(genie.QueryBatch([0, 1], [0], [0], [0], 5))
    assert list(cnt) == [1] * 5


def test_batch_submit_collect_in_turn(genie, oracle):
    """Two batches used in turn through submit / collect (the pipelined
    public path) give every query batch the oracle's results."""
    from genie_gb300 import workloads
    values, first = workloads.config1(n=20_000, d=24, q=48, k=10, buckets=64)
    t = genie.Table.from_values(values)
    ox = oracle.Index(values)
    batches = [first] + [workloads.config1_queries(values, 48, 10, buckets=64, seed=s) for s in (11, 12, 13)]
    pair = (genie.Batch(t, 48, 48 * 24, 10), genie.Batch(t, 48, 48 * 24, 10))
    expect = [ox.search(_qb(genie, b).as_oracle_batch())[:2] for b in batches]
    pend, got = [], []
    order = list(range(len(batches))) * 2
    for i, j in enumerate(order):
        b = pair[i % 2]
        if len(pend) == 2:
            bb, jj = pend.pop(0)
            got.append((jj, bb.collect()))
        b.submit(_qb(genie, batches[j]))
        pend.append((b, j))
    for bb, jj in pend:
        got.append((jj, bb.collect()))
    assert len(got) == len(order)
    for j, (ids, cnt) in got:
        assert np.array_equal(ids, expect[j][0]) and np.array_equal(cnt, expect[j][1])
