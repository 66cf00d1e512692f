"""The plugin point: a match function registered per codec id
(genie_codec_set_match, the reference's COMPRESSION_TYPE ->
MatchIntegratedFunPtr map, DeviceCodecFactory.cu:48-70) is what
genie_search and genie_search_multi call for indexes of that codec."""
import ctypes

import numpy as np
import pytest

MATCH_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.c_void_p, ctypes.c_void_p)


def test_registry_set_get_and_reject_unknown_codec():
    from genie_gb300 import build
    build.build()
    import genie_gb300 as genie
    lib = genie.lib()
    calls = []

    @MATCH_FN
    def fn(ix, q, ids, cnt, sc, user):
        calls.append(user)
        return 0

    assert lib.genie_codec_set_match(13, ctypes.cast(fn, ctypes.c_void_p), ctypes.c_void_p(77)) == 0
    got_fn, got_user = ctypes.c_void_p(), ctypes.c_void_p()
    assert lib.genie_codec_get_match(13, ctypes.byref(got_fn), ctypes.byref(got_user)) == 0
    assert got_fn.value == ctypes.cast(fn, ctypes.c_void_p).value and got_user.value == 77
    assert lib.genie_codec_set_match(13, None, None) == 0          # back to the built-in path
    assert lib.genie_codec_get_match(13, ctypes.byref(got_fn), ctypes.byref(got_user)) == 0
    assert not got_fn.value and not got_user.value
    assert lib.genie_codec_set_match(14, None, None) == 1
    assert lib.genie_codec_set_match(-1, None, None) == 1


@pytest.mark.gpu
def test_registered_match_runs_for_its_codec(genie):
    from genie_gb300 import workloads
    lib = genie.lib()
    values, b = workloads.config2(n=60_000, q=24, k=16)
    tc = genie.Table.compressed(values, 13, 128)
    tp = genie.Table.from_values(values)
    qb = genie.QueryBatch(b["item_off"], b["dim"], b["low"], b["up"], b["k"])
    want_c = genie.search(tc, qb)
    want_p = genie.search(tp, qb)
    calls = []

    @MATCH_FN
    def wrapped(ix, q, ids, cnt, sc, user):       # delegate to the built-in match and count the calls
        calls.append((ix, user))
        return lib.genie_match_builtin(ix, q, ids, cnt, sc)

    try:
        assert lib.genie_codec_set_match(13, ctypes.cast(wrapped, ctypes.c_void_p), ctypes.c_void_p(5)) == 0
        got = genie.search(tc, qb)
        assert calls == [(tc.handle.value, 5)]
        assert all(np.array_equal(w, g) for w, g in zip(want_c, got))
        genie.search(tp, qb)                          # codec 0 is not routed through it
        assert len(calls) == 1
        # multi-index search: the compressed index through the function, the plain one built in
        n = qb.total_k
        ids = np.zeros(2 * n, np.uint32)
        cnt = np.zeros(2 * n, np.uint32)
        qs = (genie._lib.GenieQueries * 2)(qb.struct(), qb.struct())
        hs = (ctypes.c_void_p * 2)(tc.handle.value, tp.handle.value)
        genie._check(lib.genie_search_multi(hs, qs, 2, ids.ctypes.data, cnt.ctypes.data, None))
        assert len(calls) == 2
        assert np.array_equal(ids[:n], want_c[0]) and np.array_equal(cnt[:n], want_c[1])
        assert np.array_equal(ids[n:], want_p[0]) and np.array_equal(cnt[n:], want_p[1])
    finally:
        lib.genie_codec_set_match(13, None, None)
