"""The CPU oracle pinned against the reference: the golden vectors of its own
tests and fixtures produced by the reference's host code (tests/golden/)."""
import json
import os
import zlib

import numpy as np
import pytest

from conftest import GOLDEN, golden


def _exact_batch(rows, d, k):
    rows = np.asarray(rows, np.int32)
    q = len(rows)
    flat = rows[:, :d].ravel()
    return dict(item_off=np.arange(q + 1) * d, dim=np.tile(np.arange(d), q), low=flat, up=flat,
                k=np.full(q, k, np.uint32))


def test_sift20_index_and_topk_goldens(oracle):
    """test/test_csv_input_sift_data.cc:65-87 (dim 5, k 5, radius 0, 3 queries)."""
    z = golden("sift20.npz")
    ix = oracle.Index(z["values"])
    assert list(ix.ids[:6]) == [8, 9, 7, 0, 2, 4]
    ids, cnt, sc, _ = ix.search(_exact_batch(z["values"][:3], 5, 5))
    assert (ids[0], cnt[0]) == (0, 5)
    assert (ids[1], cnt[1]) == (4, 2)
    assert (ids[5], cnt[5]) == (1, 5)
    assert (ids[10], cnt[10]) == (2, 5)
    # full canonical lists (count desc, id asc) recomputed by brute force
    vals = z["values"]
    for qi in range(3):
        c = (vals == vals[qi]).sum(axis=1)
        order = sorted(range(len(c)), key=lambda o: (-c[o], o))[:5]
        assert list(ids[qi * 5:(qi + 1) * 5]) == order
        assert list(cnt[qi * 5:(qi + 1) * 5]) == [c[o] for o in order]


@pytest.mark.parametrize("name", ["sift20", "sift1k", "synthetic_wide"])
def test_index_and_spans_match_reference_build(oracle, name):
    """Posting order and item spans equal the reference's inv_table / Query::build,
    including adaptive ranges (query.cc:196-261) for sift_1k_query's items."""
    z = golden(name + ".npz")
    ix = oracle.Index(z["values"])
    assert np.array_equal(ix.ids, z["inv"])
    for i in range(len(z["dim"])):
        d, lo, hi, sel = int(z["dim"][i]), int(z["low"][i]), int(z["up"][i]), float(z["sel"][i])
        if sel > 0:
            lo, hi = ix.adaptive_range(d, sel, lo, hi)
        assert ix.span(d, lo, hi) == (z["start"][i], z["end"][i]), i


def test_bag_index_matches_reference_build(oracle):
    """load_table_bijectMap (inv_list.cc:51-84): test_csv_input_tweets.cc:65-71."""
    z = golden("tweets20.npz")
    ix = oracle.Index(bag=(z["values"], z["row_off"]))
    assert np.array_equal(ix.ids, z["inv"])
    assert list(ix.ids[:6]) == [0, 11, 0, 11, 0, 11]
    for i in range(len(z["dim"])):
        assert ix.span(int(z["dim"][i]), int(z["low"][i]), int(z["up"][i])) == (z["start"][i], z["end"][i])


def test_bag_counts_do_not_wrap(oracle):
    """test_csv_input_tweets.cc:77-85 asserts count 16 for query 0: the
    reference's 4-bit bitmap counter (count_threshold 14) wraps the true count.
    The oracle counts exactly; query 1 (count 14, no wrap) agrees."""
    z = golden("tweets20.npz")
    vals, off = z["values"], z["row_off"]
    ix = oracle.Index(bag=(vals, off))
    rows = [vals[off[r]:off[r + 1]] for r in range(3)]
    item_off = np.zeros(4, np.int64)
    item_off[1:] = np.cumsum([len(r) for r in rows])
    flat = np.concatenate(rows)
    ids, cnt, _, _ = ix.search(dict(item_off=item_off, dim=np.zeros(len(flat), np.int32), low=flat, up=flat,
                                    k=np.full(3, 5, np.uint32)))
    assert ids[0] in (0, 11) and cnt[0] == 17 and cnt[1] == 17
    assert (ids[5], cnt[5]) == (1, 14)
    assert ids[10] == 2 and cnt[10] > 16


def test_codecs_match_reference_encoders(oracle):
    """All 13 reference codecs (DeviceCodecFactory.cu:13-48) on the
    test_compression_codecs.cu input stream, every length 1..1024."""
    with open(os.path.join(GOLDEN, "codecs_kat.json")) as f:
        kat = json.load(f)
    x = oracle.kat_input(1024, kat["input_seed"])
    for name, e in kat["codecs"].items():
        for n in range(1, 1025):
            w = oracle.encode(e["id"], x[:n])
            assert len(w) == e["words"][n - 1], (name, n)
            assert zlib.crc32(w.tobytes()) == e["crc32"][n - 1], (name, n)
            assert np.array_equal(oracle.decode(e["id"], w, n), x[:n]), (name, n)
        for n, words in e["full"].items():
            assert list(oracle.encode(e["id"], x[:int(n)])) == words


def test_weighted_scores_close_to_fp64(oracle):
    rng = np.random.default_rng(7)
    vals = rng.integers(0, 6, size=(3000, 24)).astype(np.int32)
    ix = oracle.Index(vals)
    q = 40
    m = 24
    flat = rng.integers(0, 6, size=q * m).astype(np.int32)
    w = rng.uniform(0.5, 2.0, q * m).astype(np.float32)
    b = dict(item_off=np.arange(q + 1) * m, dim=np.tile(np.arange(m), q), low=flat, up=flat,
             k=np.full(q, 50, np.uint32), weight=w, weighted=np.ones(q, np.uint8))
    ids, cnt, sc, _ = ix.search(b)
    for qi in range(q):
        qw = w[qi * m:(qi + 1) * m].astype(np.float64)
        qv = flat[qi * m:(qi + 1) * m]
        s64 = ((vals == qv) * qw).sum(axis=1)
        got = ids[qi * 50:(qi + 1) * 50]
        ref = s64[got]
        assert np.all(np.abs(sc[qi * 50:(qi + 1) * 50] - ref) <= 1e-6 * ref)
        # the returned set is the top 50 of the FP64 scores (no near-ties at the cut here)
        best = np.sort(s64)[::-1][:50]
        assert np.allclose(np.sort(ref)[::-1], best, rtol=1e-6)


def test_empty_and_out_of_range_items(oracle):
    vals = np.arange(20, dtype=np.int32).reshape(10, 2)
    ix = oracle.Index(vals)
    b = dict(item_off=np.array([0, 0, 3, 4]), dim=np.array([-1, 2, 0, 1]), low=np.array([0, 0, 5, 9]),
             up=np.array([100, 100, 4, 9]), k=np.array([3, 3, 3], np.uint32))
    ids, cnt, _, _ = ix.search(b)
    assert list(cnt[:6]) == [0] * 6 and list(ids[:6]) == [0] * 6
    assert (ids[6], cnt[6]) == (4, 1) and cnt[7] == 0
