"""The dense kernel's list access paths against the oracle: tile cuts from the
index's tile directory or from searches, dense lists counted from their
presence bitmaps or from their ids, single- and multi-chunk queries (more
list units than one staged chunk), weighted and unweighted counters."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _qb(genie, b):
    return genie.QueryBatch(b["item_off"], b["dim"], b["low"], b["up"], b["k"], b.get("weight"), b.get("weighted"))


@pytest.mark.parametrize("tiles", [
    dict(dense_bitmaps=3),                          # default tiles: directories and bitmaps
    dict(dense_bitmaps=-1),                         # directories, every list from its ids
    dict(dense_tile=40016, dense_bitmaps=2),        # another tile size, bitmaps for weighted queries only
    dict(dense_tile=65536, dense_bitmaps=1),        # other directory sizes, bitmaps for bytes only
    dict(dense_tile=40016, dense_part_work=3 * 40016),  # parts of several tiles (running top-k across tiles)
    dict(dense_tile=65536, dense_part_work=1, dense_bitmaps=3),  # below one tile: one tile per part
])
def test_dense_paths_equal_oracle(genie, oracle, tiles):
    from genie_gb300 import workloads
    values, b = workloads.config3(n=260_000, q=40, min_items=40, max_items=128)
    # half the queries with radius 4 over many items: more list units than one chunk
    b["low"] = np.where(np.repeat(np.arange(40) % 2 == 0, np.diff(b["item_off"])), b["low"] - 4, b["low"])
    t = genie.Table.from_values(values)
    qb = _qb(genie, b)
    bt = genie.Batch(t, qb.n_queries, len(b["dim"]), 100, use_graph=False)
    bt.set_tuning(sparse_max_total=1, bitmap_bits=-1, **tiles)
    ids, cnt, sc = bt.run(qb, scores=True)
    oid, ocnt, osc, _ = oracle.Index(values).search(qb.as_oracle_batch())
    assert np.array_equal(cnt, ocnt) and np.array_equal(ids, oid) and np.array_equal(sc, osc)
    # the plain path (its own workspace, default tuning) agrees
    pid, pcnt, psc = genie.search(t, qb, scores=True)
    assert np.array_equal(pid, oid) and np.array_equal(pcnt, ocnt) and np.array_equal(psc, osc)
