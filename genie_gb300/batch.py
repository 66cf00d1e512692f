"""Batched search handle (genie_batch_*): fixed-capacity device buffers,
pinned staging, device-side query compile, persistent kernels in one CUDA
graph, and the autotuner."""
import ctypes

import numpy as np

from . import _lib


class Batch:
    def __init__(self, table, max_queries, max_items, max_k, use_graph=True, max_units=0):
        from . import _check, lib
        cfg = _lib.GenieBatchConfig(int(max_queries), int(max_items), int(max_k), int(bool(use_graph)),
                                    int(max_units))
        h = ctypes.c_void_p()
        _check(lib().genie_batch_create(table.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.table = table
        self._staged = None

    def _outs(self, n, scores):
        ids = np.zeros(max(1, n), np.uint32)
        cnt = np.zeros(max(1, n), np.uint32)
        sc = np.zeros(max(1, n), np.float32) if scores else None
        return ids, cnt, sc

    def run(self, batch, scores=False):
        """stage + launch + fetch (synchronous)."""
        from . import _check, lib
        n = batch.total_k
        ids, cnt, sc = self._outs(n, scores)
        s = batch.struct()
        _check(lib().genie_batch_run(self._h, ctypes.byref(s), ids.ctypes.data, cnt.ctypes.data,
                                     None if sc is None else sc.ctypes.data))
        self._staged = batch
        return (ids[:n], cnt[:n], sc[:n]) if scores else (ids[:n], cnt[:n])

    def stage(self, batch):
        from . import _check, lib
        s = batch.struct()
        _check(lib().genie_batch_stage(self._h, ctypes.byref(s)))
        self._staged = batch

    def launch(self, stream=None):
        """Enqueue the device work of the staged batch on a cudaStream_t (int)."""
        from . import _check, lib
        _check(lib().genie_batch_launch(self._h, None if stream is None else ctypes.c_void_p(stream)))

    def fetch(self, scores=False):
        from . import _check, lib
        n = self._staged.total_k
        ids, cnt, sc = self._outs(n, scores)
        _check(lib().genie_batch_fetch(self._h, ids.ctypes.data, cnt.ctypes.data,
                                       None if sc is None else sc.ctypes.data))
        return (ids[:n], cnt[:n], sc[:n]) if scores else (ids[:n], cnt[:n])

    def submit(self, batch, scores=False):
        """Asynchronous run: stage `batch`, enqueue its device work and result
        download, and return; collect() waits and returns the results.  Two
        batches used in turn overlap host staging with device work."""
        from . import _check, lib
        s = batch.struct()
        _check(lib().genie_batch_submit(self._h, ctypes.byref(s), 1 if scores else 0))
        self._staged = batch
        self._submitted_scores = scores

    def collect(self):
        from . import _check, lib
        scores = getattr(self, "_submitted_scores", False)
        n = self._staged.total_k
        ids, cnt, sc = self._outs(n, scores)
        _check(lib().genie_batch_collect(self._h, ids.ctypes.data, cnt.ctypes.data,
                                         None if sc is None else sc.ctypes.data))
        return (ids[:n], cnt[:n], sc[:n]) if scores else (ids[:n], cnt[:n])

    def autotune(self, sample):
        from . import _check, lib
        t = _lib.GenieTuning()
        s = sample.struct()
        _check(lib().genie_batch_autotune(self._h, ctypes.byref(s), ctypes.byref(t)))
        self._staged = sample
        return {f: getattr(t, f) for f, _ in _lib.GenieTuning._fields_}

    def tuning(self):
        from . import _check, lib
        t = _lib.GenieTuning()
        _check(lib().genie_batch_get_tuning(self._h, ctypes.byref(t)))
        return {f: getattr(t, f) for f, _ in _lib.GenieTuning._fields_}

    def set_tuning(self, **kw):
        from . import _check, lib
        t = _lib.GenieTuning()
        for k, v in kw.items():
            setattr(t, k, v)
        _check(lib().genie_batch_set_tuning(self._h, ctypes.byref(t)))

    def last_stats(self):
        from . import _check, lib
        k = ctypes.c_int32()
        ms = ctypes.c_float()
        _check(lib().genie_batch_last_stats(self._h, ctypes.byref(k), ctypes.byref(ms)))
        return k.value, ms.value

    def stage_ms(self):
        """Per-stage device ms of the last launch (batches made with use_graph=False):
        plan, bitmap, sparse (both slot widths), dense (both counter widths)."""
        from . import _check, lib
        ms = np.zeros(4, np.float32)
        _check(lib().genie_batch_stage_ms(self._h, ms.ctypes.data))
        return ms

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
