"""The request protocol over the serving loop (dist_genie's JSON
{topk, queries: [{content, clusters}]} requests, parser.cu:128-216, one per
TCP connection, scheduler.cc:20-64): validation messages and the socket
loop on the CPU; searches merged over clusters against the oracle on the GPU."""
import ctypes
import json
import socket

import numpy as np
import pytest


def _lib():
    from genie_gb300 import build
    build.build()
    import genie_gb300 as g
    return g


def _router(g, server, index_ids, offsets, radius=0):
    ids = (ctypes.c_int32 * len(index_ids))(*index_ids)
    offs = (ctypes.c_int64 * len(offsets))(*offsets)
    r = g._lib.GenieRequestRouter(server, len(index_ids), ctypes.cast(ids, ctypes.c_void_p),
                                  ctypes.cast(offs, ctypes.c_void_p), radius)
    r._keep = (ids, offs)
    return r


def _handle(g, router, doc):
    buf = ctypes.create_string_buffer(1 << 20)
    n = ctypes.c_int64()
    g._check(g.lib().genie_request_handle(ctypes.byref(router), doc.encode(), buf, len(buf), ctypes.byref(n)))
    return json.loads(buf.value.decode())


def _send(port, doc):
    with socket.create_connection(("127.0.0.1", port), timeout=60) as s:
        s.sendall(doc.encode())
        s.shutdown(socket.SHUT_WR)
        chunks = []
        while True:
            b = s.recv(65536)
            if not b:
                break
            chunks.append(b)
    return json.loads(b"".join(chunks).decode())


BAD = [
    ("{not json", "Received query is not a valid JSON document"),
    ('{"queries": []}', "Entry 'topk' is missing"),
    ('{"topk": 1.5, "queries": []}', "Entry 'topk' should be an interger"),
    ('{"topk": 5}', "Entry 'queries' is missing"),
    ('{"topk": 5, "queries": {}}', "Entry 'queries' should be an array"),
    ('{"topk": 5, "queries": [{"clusters": [0]}]}', "Some query misses the 'content' section"),
    ('{"topk": 5, "queries": [{"content": 3, "clusters": [0]}]}', "Query's 'content' section should be an array"),
    ('{"topk": 5, "queries": [{"content": [1]}]}', "Some query misses the 'clusters' section"),
    ('{"topk": 5, "queries": [{"content": [1], "clusters": 0}]}', "Query's 'clusters' section should be an array"),
    ('{"topk": 5, "queries": [{"content": [1], "clusters": [7]}]}', "Query's 'clusters' should name clusters 0..1"),
]


@pytest.mark.parametrize("doc,msg", BAD)
def test_request_validation_messages(doc, msg):
    g = _lib()
    router = _router(g, None, [0, 1], [0, 100])
    assert _handle(g, router, doc) == {"error": msg}


def test_listener_answers_each_connection_on_the_cpu():
    g = _lib()
    router = _router(g, None, [0, 1], [0, 100])
    lis = ctypes.c_void_p()
    g._check(g.lib().genie_request_listen(ctypes.byref(router), b"127.0.0.1", 0, ctypes.byref(lis)))
    try:
        port = ctypes.c_int32()
        g._check(g.lib().genie_request_listener_port(lis, ctypes.byref(port)))
        assert port.value > 0
        assert _send(port.value, "{oops") == {"error": "Received query is not a valid JSON document"}
        assert _send(port.value, '{"topk": 3, "queries": [{"content": [1], "clusters": [0]}]}') == \
            {"error": "no server attached"}
        n = ctypes.c_int64()
        g._check(g.lib().genie_request_listener_handled(lis, ctypes.byref(n)))
        assert n.value == 2
    finally:
        g.lib().genie_request_listener_stop(lis)


@pytest.mark.gpu
def test_requests_search_and_merge_clusters(genie, oracle):
    """Two clusters (the halves of one table) behind a server: each query's
    answer over the clusters it names equals the oracle's over those rows,
    with global ids."""
    from genie_gb300 import workloads
    values, b = workloads.config0(n=4000, q=12, k=10)
    half = 2000
    ta = genie.Table.from_values(values[:half])
    tb = genie.Table.from_values(values[half:])
    srv = genie.Server(max_queries=16, max_items=16 * 128, max_k=32, slots_per_index=2, window_us=50)
    ia, ib = srv.add_index(ta), srv.add_index(tb)
    srv.start()
    router = _router(genie, srv._h, [ia, ib], [0, half], radius=1)
    lis = ctypes.c_void_p()
    genie._check(genie.lib().genie_request_listen(ctypes.byref(router), b"127.0.0.1", 0, ctypes.byref(lis)))
    try:
        port = ctypes.c_int32()
        genie._check(genie.lib().genie_request_listener_port(lis, ctypes.byref(port)))
        d = values.shape[1]
        qv = [b["low"][i * d:(i + 1) * d].tolist() for i in range(12)]
        which = [[0], [1], [0, 1]] * 4
        req = {"topk": 10, "queries": [{"content": qv[i], "clusters": which[i]} for i in range(12)]}
        got = _send(port.value, json.dumps(req))
        assert got["topk"] == 10 and len(got["results"]) == 12
        for i in range(12):
            rows = np.concatenate([np.arange(half) if c == 0 else np.arange(half, 4000) for c in which[i]])
            ox = oracle.Index(values[rows])
            flat = np.array(qv[i], np.int32)
            batch = dict(item_off=np.array([0, d]), dim=np.arange(d, dtype=np.int32), low=flat - 1, up=flat + 1,
                         k=np.array([10], np.uint32))
            oid, ocnt, _, _ = ox.search(batch)
            want_ids = np.where(ocnt > 0, rows[oid], 0)
            assert got["results"][i]["counts"] == ocnt.tolist(), i
            assert got["results"][i]["ids"] == want_ids.tolist(), i
    finally:
        genie.lib().genie_request_listener_stop(lis)
        srv.close()
