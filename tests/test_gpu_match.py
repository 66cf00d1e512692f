"""CUDA match path vs the CPU oracle, through the C ABI.

Unweighted ids/counts and weighted ids are bit-exact; weighted scores equal
the oracle's (same exact fixed-point sum, one rounding) and lie within 1e-6
relative of an FP64 recompute (checked in test_oracle_golden)."""
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _check(genie, oracle, values, batch, bag=None, scores=True):
    if bag is not None:
        t = genie.Table.from_bag_arrays(*bag)
        ox = oracle.Index(bag=bag)
    else:
        t = genie.Table.from_values(values)
        ox = oracle.Index(values)
    qb = genie.QueryBatch(batch["item_off"], batch["dim"], batch["low"], batch["up"], batch["k"],
                          batch.get("weight"), batch.get("weighted"))
    ids, cnt, sc = genie.search(t, qb, scores=True)
    oid, ocnt, osc, _ = ox.search(qb.as_oracle_batch())
    assert np.array_equal(cnt, ocnt)
    assert np.array_equal(ids, oid)
    if scores:
        assert np.array_equal(sc, osc)
    return t, ids, cnt, sc


def test_sift20_goldens_first_level_interface(genie, tmp_path):
    """genie::Search over sift_20 (test_refactoring_new_interface.cc:22-38,
    test_csv_input_sift_data.cc:65-87)."""
    z = golden("sift20.npz")
    p = tmp_path / "sift_20.csv"
    with open(p, "w") as f:
        for row in z["values"]:
            f.write(",".join(str(v) for v in row) + ",\n")
    policy = genie.MakePolicy(genie.Config().SetK(5).SetNumOfQueries(3))
    ids, counts = genie.Search(policy, str(p), str(p))
    assert len(ids) == 15
    assert (ids[0], counts[0]) == (0, 5)
    assert (ids[1], counts[1]) == (4, 2)
    assert (ids[5], counts[5]) == (1, 5)
    assert (ids[10], counts[10]) == (2, 5)
    assert ids[:5] == [0, 4, 2, 6, 9] and counts[:5] == [5, 2, 1, 1, 1]


def test_device_postings_equal_reference_inv(genie):
    """test_save2gpu_sift.cc:91-100: the device posting array equals _inv."""
    for name in ("sift20", "sift1k", "synthetic_wide"):
        z = golden(name + ".npz")
        t = genie.Table.from_values(z["values"])
        assert np.array_equal(t.inv(), z["inv"]), name
        for i in range(0, len(z["dim"]), 7):
            if z["sel"][i] > 0:
                continue
            assert t.span(int(z["dim"][i]), int(z["low"][i]), int(z["up"][i])) == (z["start"][i], z["end"][i])


def test_config0_exact(genie, oracle):
    from genie_gb300 import workloads
    values, batch = workloads.config0()
    _check(genie, oracle, values, batch)


def test_sift1k_multirange_adaptive(genie, oracle):
    """sift_1k_query.csv (qid, dim, value, sel 0.04, weight 1) through the
    adaptive range, k=10, against the oracle."""
    z = golden("sift1k.npz")
    mq = np.load(os.path.join(os.path.dirname(__file__), "golden", "sift1k_multirange.npy"))
    t = genie.Table.from_values(z["values"])
    qids = np.unique(mq[:, 0])
    off, dims, lows, ups = [0], [], [], []
    for qid in qids:
        rows = mq[mq[:, 0] == qid]
        for _, d, v in rows:
            lo, hi = t.adaptive_range(int(d), 0.04, int(v), int(v))
            dims.append(d); lows.append(lo); ups.append(hi)
        off.append(len(dims))
    batch = dict(item_off=np.array(off), dim=np.array(dims), low=np.array(lows), up=np.array(ups),
                 k=np.full(len(qids), 10, np.uint32))
    _check(genie, oracle, z["values"], batch)


def test_config1_shape_sparse(genie, oracle):
    from genie_gb300 import workloads
    values, batch = workloads.config1(n=200_000, q=192, k=100)
    _check(genie, oracle, values, batch)


def test_sparse_multi_part_and_wide_entries(genie, oracle):
    rng = np.random.default_rng(3)
    values = rng.integers(0, 256, size=(1_000_000, 16), dtype=np.int32)
    q = 24
    flat = rng.integers(0, 256, size=q * 16).astype(np.int32)
    batch = dict(item_off=np.arange(q + 1) * 16, dim=np.tile(np.arange(16), q), low=flat, up=flat,
                 k=np.full(q, 64, np.uint32))
    _check(genie, oracle, values, batch)          # ~62K touched ids: 4 hash parts
    w = rng.uniform(0.5, 2.0, q * 16).astype(np.float32)
    batch.update(weight=w, weighted=(np.arange(q) % 2).astype(np.uint8))
    _check(genie, oracle, values, batch)          # weighted queries use 8-byte slots


def test_sparse_overflow_retries_dense(genie, oracle):
    """Touched ids concentrated in one id-range part overflow its hash; the
    query is redone by the dense kernel (the reference grows its hash table
    and relaunches, match.cu:356-421)."""
    n = 1_000_000
    values = np.zeros((n, 4), np.int32)
    values[:25_000, :] = 7
    values[25_000:, :] = np.random.default_rng(5).integers(8, 100, size=(n - 25_000, 4))
    batch = dict(item_off=np.array([0, 4, 8]), dim=np.array([0, 1, 2, 3, 0, 1, 2, 3]),
                 low=np.array([7, 7, 7, 7, 7, 7, 7, 50]), up=np.array([7, 7, 7, 7, 7, 7, 7, 60]),
                 k=np.array([100, 2048], np.uint32))
    _check(genie, oracle, values, batch)


def test_config3_shape_mixed(genie, oracle):
    from genie_gb300 import workloads
    values, batch = workloads.config3(n=300_000, q=96)
    _check(genie, oracle, values, batch)


def test_dense_multi_part(genie, oracle):
    rng = np.random.default_rng(11)
    values = rng.integers(0, 8, size=(2_000_000, 32), dtype=np.int32)
    q = 4
    flat = rng.integers(0, 8, size=q * 32).astype(np.int32)
    batch = dict(item_off=np.arange(q + 1) * 32, dim=np.tile(np.arange(32), q), low=flat, up=flat,
                 k=np.array([1, 10, 500, 2048], np.uint32))
    _check(genie, oracle, values, batch)


def test_many_items_and_large_counts(genie, oracle):
    """More than 512 items per query (staged in chunks) and counts above 255
    (4-byte counters)."""
    rng = np.random.default_rng(2)
    values = rng.integers(0, 4, size=(20_000, 300), dtype=np.int32)
    q = 6
    m = 600
    dims = np.concatenate([rng.integers(0, 300, m) for _ in range(q)]).astype(np.int32)
    lo = rng.integers(0, 4, q * m).astype(np.int32)
    batch = dict(item_off=np.arange(q + 1) * m, dim=dims, low=lo, up=lo + 1, k=np.full(q, 30, np.uint32))
    _check(genie, oracle, values, batch)


def test_bag_index_search(genie, oracle):
    z = golden("tweets20.npz")
    vals, off = z["values"], z["row_off"]
    rows = [vals[off[r]:off[r + 1]] for r in range(5)]
    item_off = np.zeros(6, np.int64)
    item_off[1:] = np.cumsum([len(r) for r in rows])
    flat = np.concatenate(rows)
    batch = dict(item_off=item_off, dim=np.zeros(len(flat), np.int32), low=flat, up=flat,
                 k=np.full(5, 5, np.uint32))
    _, ids, cnt, _ = _check(genie, oracle, None, batch, bag=(vals, off))
    assert ids[0] in (0, 11) and cnt[0] == 17       # exact, where the reference wraps to 16
    # random bags with repeated words
    rng = np.random.default_rng(9)
    lens = rng.integers(1, 30, 5000)
    roff = np.zeros(5001, np.int64)
    roff[1:] = np.cumsum(lens)
    words = rng.integers(0, 500, roff[-1]).astype(np.int32)
    qlen = rng.integers(1, 40, 50)
    qoff = np.zeros(51, np.int64)
    qoff[1:] = np.cumsum(qlen)
    qw = rng.integers(0, 520, qoff[-1]).astype(np.int32)
    batch = dict(item_off=qoff, dim=np.zeros(qoff[-1], np.int32), low=qw, up=qw + rng.integers(0, 2, qoff[-1]),
                 k=np.full(50, 20, np.uint32))
    _check(genie, oracle, None, batch, bag=(words, roff))


def test_edge_cases(genie, oracle):
    values = np.arange(40, dtype=np.int32).reshape(20, 2) % 7
    batch = dict(item_off=np.array([0, 0, 3, 5, 6]), dim=np.array([-1, 2, 0, 1, 1, 0]),
                 low=np.array([0, 0, 5, 9, 3, -50]), up=np.array([100, 100, 4, 2, 3, 50]),
                 k=np.array([3, 3, 30, 1], np.uint32))
    _check(genie, oracle, values, batch)
    one = np.array([[5, 6, 7]], np.int32)
    _check(genie, oracle, one, dict(item_off=np.array([0, 3]), dim=np.array([0, 1, 2]), low=np.array([5, 6, 0]),
                                    up=np.array([5, 6, 0]), k=np.array([4], np.uint32)))


def test_invalid_arguments(genie):
    t = genie.Table.from_values(np.zeros((10, 2), np.int32))
    ok = dict(item_off=[0, 1], dim=[0], low=[0], up=[0])
    with pytest.raises(genie.cpu_runtime_error):
        genie.search(t, genie.QueryBatch(k=0, **ok))
    with pytest.raises(genie.cpu_runtime_error):
        genie.search(t, genie.QueryBatch(k=4096, **ok))
    with pytest.raises(genie.cpu_runtime_error):
        genie.search(t, genie.QueryBatch(k=1, weight=[-1.0], weighted=[1], **ok))
    with pytest.raises(genie.cpu_runtime_error):
        genie.search(t, genie.QueryBatch(k=1, weight=[float("nan")], weighted=[1], **ok))
    # the handle stays usable after rejected calls
    ids, cnt = genie.search(t, genie.QueryBatch(k=2, **ok))
    assert list(cnt) == [1, 1] and list(ids) == [0, 1]


def test_save_load_roundtrip(genie, oracle, tmp_path):
    from genie_gb300 import workloads
    values, batch = workloads.config0(n=3000, q=20)
    t = genie.Table.from_values(values)
    p = str(tmp_path / "ix.genie")
    genie.SaveTableToBinary(p, t)
    t2 = genie.LoadTableFromBinary(p)
    assert np.array_equal(t2.inv(), t.inv())
    qb = genie.QueryBatch(batch["item_off"], batch["dim"], batch["low"], batch["up"], batch["k"])
    assert all(np.array_equal(a, b) for a, b in zip(genie.search(t, qb), genie.search(t2, qb)))
    raw = bytearray(open(p, "rb").read())
    raw[200] ^= 0xFF
    bad = str(tmp_path / "bad.genie")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(genie.cpu_runtime_error):
        genie.LoadTableFromBinary(bad)
    open(bad, "wb").write(bytes(raw[:100]))
    with pytest.raises(genie.cpu_runtime_error):
        genie.LoadTableFromBinary(bad)


def test_multi_index_search(genie, oracle):
    """knn_search_MT: several resident tables searched together."""
    import ctypes
    from genie_gb300 import workloads
    tabs, batches, expect = [], [], []
    for i, n in enumerate((2000, 5000, 800)):
        values, batch = workloads.config0(n=n, q=10 + i, k=5 + i, seed=100 + i)
        tabs.append(genie.Table.from_values(values))
        qb = genie.QueryBatch(batch["item_off"], batch["dim"], batch["low"], batch["up"], batch["k"])
        batches.append(qb)
        expect.append(oracle.Index(values).search(qb.as_oracle_batch()))
    tot = sum(b.total_k for b in batches)
    ids = np.zeros(tot, np.uint32)
    cnt = np.zeros(tot, np.uint32)
    hs = (ctypes.c_void_p * 3)(*[t.handle.value for t in tabs])
    qs = (genie._lib.GenieQueries * 3)(*[b.struct() for b in batches])
    genie._check(genie.lib().genie_search_multi(hs, qs, 3, ids.ctypes.data, cnt.ctypes.data, None))
    o = 0
    for b, e in zip(batches, expect):
        assert np.array_equal(ids[o:o + b.total_k], e[0])
        assert np.array_equal(cnt[o:o + b.total_k], e[1])
        o += b.total_k
