"""Device decoders and compressed-index search.

test_compression_codecs.cu: every codec round-trips lengths 1..1024 of the
srand(666) stream (host encode -> GPU decode == input).
test_compression_kernels.cu: search over a compressed table equals search
over the uncompressed one, for every codec."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _encode(lib, codec, x):
    cap = lib.genie_codec_encode_bound(len(x))
    out = np.zeros(cap, np.uint32)
    n = lib.genie_codec_encode(codec, np.ascontiguousarray(x, np.uint32).ctypes.data, len(x), out.ctypes.data, cap)
    assert n > 0
    return out[:n]


def test_device_decode_all_codecs_all_lengths(genie, oracle):
    import torch
    lib = genie.lib()
    x = oracle.kat_input(1024)
    for name, codec in oracle.CODECS.items():
        segs = [_encode(lib, codec, x[:n]) for n in range(1, 1025)]
        woff = np.zeros(1025, np.int64)
        woff[1:] = np.cumsum([len(s) for s in segs])
        ooff = np.zeros(1025, np.int64)
        ooff[1:] = np.cumsum(np.arange(1, 1025))
        words = torch.from_numpy(np.concatenate(segs).view(np.int32)).cuda()
        d_woff = torch.from_numpy(woff).cuda()
        d_ooff = torch.from_numpy(ooff).cuda()
        out = torch.zeros(int(ooff[-1]) + 64, dtype=torch.int32, device="cuda")
        out_len = torch.zeros(1024, dtype=torch.int32, device="cuda")
        genie._check(lib.genie_codec_decode_device(codec, words.data_ptr(), d_woff.data_ptr(), 1024,
                                                   d_ooff.data_ptr(), out.data_ptr(), out_len.data_ptr(), None))
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        lens = out_len.cpu().numpy()
        assert np.array_equal(lens, np.arange(1, 1025)), name
        for n in range(1, 1025):
            assert np.array_equal(got[ooff[n - 1]:ooff[n]], x[:n]), (name, n)


def _zipf_table(n, d, terms, seed):
    from genie_gb300 import workloads
    rng = np.random.default_rng(seed)
    values = workloads.zipf_ranks(rng, (n, d), n_terms=terms)
    q = 24
    qv = workloads.zipf_ranks(rng, (q, d), n_terms=terms)
    dims = np.tile(np.arange(d), q)
    low = qv.ravel()
    up = low + rng.choice([0, 0, 0, 1, 3], q * d)
    w = rng.uniform(0.5, 2.0, q * d).astype(np.float32)
    batch = dict(item_off=np.arange(q + 1) * d, dim=dims, low=low, up=up,
                 k=rng.choice([1, 10, 32, 300], q).astype(np.uint32), weight=w,
                 weighted=(np.arange(q) % 3 == 0).astype(np.uint8))
    return values, batch


@pytest.mark.parametrize("codec", list(range(1, 14)))
def test_compressed_search_matches_oracle(genie, oracle, codec):
    values, batch = _zipf_table(60_000, 8, 2000, 40 + codec)
    t = genie.Table.compressed(values, codec, 1024)
    ox = oracle.Index(values)
    # the layout is the reference's per-segment encoding
    lay = t.compressed_layout()
    ref = ox.compress(codec, 1024)
    assert np.array_equal(lay["words"], ref["words"])
    assert np.array_equal(lay["seg_len"], ref["seg_len"]) and np.array_equal(lay["key_seg"], ref["key_seg"])
    qb = genie.QueryBatch(batch["item_off"], batch["dim"], batch["low"], batch["up"], batch["k"],
                          batch["weight"], batch["weighted"])
    ids, cnt, sc = genie.search(t, qb, scores=True)
    oid, ocnt, osc, _ = ox.search(qb.as_oracle_batch())
    assert np.array_equal(cnt, ocnt) and np.array_equal(ids, oid) and np.array_equal(sc, osc)


def test_compressed_short_segments_and_batch(genie, oracle):
    """BP32 blocks of 128 with varint tails (segments of 128 ids), through the
    batched graph path; the saved file reloads to the same answers."""
    import tempfile
    import os
    values, batch = _zipf_table(200_000, 16, 4000, 7)
    t = genie.Table.compressed(values, 13, 128)
    qb = genie.QueryBatch(batch["item_off"], batch["dim"], batch["low"], batch["up"], batch["k"],
                          batch["weight"], batch["weighted"])
    bt = genie.Batch(t, qb.n_queries, len(batch["dim"]), 300)
    ids, cnt = bt.run(qb)
    oid, ocnt, _, _ = oracle.Index(values).search(qb.as_oracle_batch())
    assert np.array_equal(cnt, ocnt) and np.array_equal(ids, oid)
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "c.genie")
        t.save(p)
        t2 = genie.Table.load(p)
        ids2, cnt2 = genie.search(t2, qb)
        assert np.array_equal(ids2, oid) and np.array_equal(cnt2, ocnt)


@pytest.mark.parametrize("codec", [3, 11, 12, 13])
def test_bp32_block_segments_dense_exact(genie, oracle, codec):
    """Full 128-id segments of the BP32-based codecs are unpacked by the dense
    kernel's word-level path (list tails by the generic decoder): every query
    forced onto the dense kernel, weighted and not, equals the oracle."""
    values, batch = _zipf_table(300_000, 8, 1500, 90 + codec)
    t = genie.Table.compressed(values, codec, 128)
    qb = genie.QueryBatch(batch["item_off"], batch["dim"], batch["low"], batch["up"], batch["k"],
                          batch["weight"], batch["weighted"])
    bt = genie.Batch(t, qb.n_queries, len(batch["dim"]), 300, use_graph=False)
    bt.set_tuning(sparse_max_total=1, bitmap_bits=-1)
    ids, cnt, sc = bt.run(qb, scores=True)
    oid, ocnt, osc, _ = oracle.Index(values).search(qb.as_oracle_batch())
    assert np.array_equal(cnt, ocnt) and np.array_equal(ids, oid) and np.array_equal(sc, osc)
    # parts of several tiles: a segment straddling a tile bound is cut in both
    bt.set_tuning(dense_tile=16384, dense_part_work=4 * 16384)
    ids, cnt, sc = bt.run(qb, scores=True)
    assert np.array_equal(cnt, ocnt) and np.array_equal(ids, oid) and np.array_equal(sc, osc)
