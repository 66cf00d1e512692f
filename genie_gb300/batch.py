"""Batched search handle (genie_batch_*): fixed-capacity device buffers,
device-side query compile, persistent kernels in one CUDA graph."""
import ctypes

import numpy as np

from . import _lib


class Batch:
    def __init__(self, table, max_queries, max_items, max_k, use_graph=True, autotune=False):
        from . import _check, lib
        cfg = _lib.GenieBatchConfig(int(max_queries), int(max_items), int(max_k), int(bool(use_graph)),
                                    int(bool(autotune)))
        h = ctypes.c_void_p()
        _check(lib().genie_batch_create(table.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.table = table

    def run(self, batch, scores=False):
        from . import _check, lib
        n = batch.total_k
        ids = np.zeros(max(1, n), np.uint32)
        cnt = np.zeros(max(1, n), np.uint32)
        sc = np.zeros(max(1, n), np.float32) if scores else None
        s = batch.struct()
        _check(lib().genie_batch_run(self._h, ctypes.byref(s), ids.ctypes.data, cnt.ctypes.data,
                                     None if sc is None else sc.ctypes.data))
        if scores:
            return ids[:n], cnt[:n], sc[:n]
        return ids[:n], cnt[:n]

    def autotune(self, sample):
        from . import _check, lib
        t = _lib.GenieTuning()
        s = sample.struct()
        _check(lib().genie_batch_autotune(self._h, ctypes.byref(s), ctypes.byref(t)))
        return {f: getattr(t, f) for f, _ in _lib.GenieTuning._fields_}

    def last_stats(self):
        from . import _check, lib
        k = ctypes.c_int32()
        ms = ctypes.c_float()
        _check(lib().genie_batch_last_stats(self._h, ctypes.byref(k), ctypes.byref(ms)))
        return k.value, ms.value

    def close(self):
        from . import lib
        if self._h is not None and self._h.value:
            lib().genie_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
