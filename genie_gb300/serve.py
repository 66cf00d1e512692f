"""Serving handle (genie_server_*): several resident indexes, admission by a
memory estimate and free batch slots, continuous batching, p50/p99 latency.

    srv = Server(max_queries=256, max_items=65536, max_k=128, slots_per_index=2)
    a = srv.add_index(table_a)
    srv.start()
    first = srv.submit(a, query_batch)            # one request per query
    ids, counts, scores, latency_ns = srv.wait(first, k)
"""
import ctypes

import numpy as np

from . import _lib


class Server:
    def __init__(self, max_queries=256, max_items=1 << 16, max_k=128, slots_per_index=2, window_us=50,
                 memory_budget=0):
        from . import _check, lib
        cfg = _lib.GenieServerConfig(int(slots_per_index), int(max_queries), int(max_items), int(max_k),
                                     int(window_us), int(memory_budget))
        h = ctypes.c_void_p()
        _check(lib().genie_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.tables = []

    def add_index(self, table):
        from . import _check, lib
        i = ctypes.c_int32()
        _check(lib().genie_server_add_index(self._h, table.handle, ctypes.byref(i)))
        self.tables.append(table)
        return i.value

    def start(self):
        from . import _check, lib
        _check(lib().genie_server_start(self._h))

    @staticmethod
    def now_ns():
        from . import lib
        return int(lib().genie_server_now_ns())

    def submit(self, index_id, batch, arrival_ns=None):
        """Submit every query of `batch` as a request.  arrival_ns: None (now),
        one time for all, or one time per query, on the server clock.
        Returns the first ticket (then +1 per query)."""
        from . import _check, lib
        s = batch.struct()
        t = ctypes.c_uint64()
        arr = None
        if arrival_ns is not None:
            arr = np.ascontiguousarray(np.broadcast_to(np.asarray(arrival_ns, np.int64), (batch.n_queries,)))
        _check(lib().genie_server_submit(self._h, int(index_id), ctypes.byref(s),
                                         None if arr is None else arr.ctypes.data, ctypes.byref(t)))
        return t.value

    def wait(self, ticket, k):
        from . import _check, lib
        ids = np.zeros(max(1, k), np.uint32)
        cnt = np.zeros(max(1, k), np.uint32)
        sc = np.zeros(max(1, k), np.float32)
        lat = ctypes.c_int64()
        _check(lib().genie_server_wait(self._h, ctypes.c_uint64(ticket), ids.ctypes.data, cnt.ctypes.data,
                                       sc.ctypes.data, ctypes.byref(lat)))
        return ids[:k], cnt[:k], sc[:k], lat.value

    def drain(self):
        from . import _check, lib
        _check(lib().genie_server_drain(self._h))

    def stats(self):
        from . import _check, lib
        r = _lib.GenieServerReport()
        _check(lib().genie_server_stats(self._h, ctypes.byref(r)))
        return {f: getattr(r, f) for f, _ in _lib.GenieServerReport._fields_}

    def reset_stats(self):
        from . import _check, lib
        _check(lib().genie_server_reset_stats(self._h))

    def close(self):
        from . import lib
        if getattr(self, "_h", None) and self._h.value:
            lib().genie_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_arrivals(rate_qps, n, seed=0, start_ns=0):
    """Open-loop Poisson arrival times (ns) of n requests at rate_qps."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1e9 / float(rate_qps), n)
    return (start_ns + np.cumsum(gaps)).astype(np.int64)
