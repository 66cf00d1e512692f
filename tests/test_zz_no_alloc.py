"""genie_search_noalloc: the search for callers that may not allocate device
memory (a framework that owns every allocation, a hard memory budget, or a
latency-critical path where cudaMalloc's device-wide synchronisation is not
acceptable).  Its workspace is a fixed array inside the library, so its
results must equal genie_search's on consecutive calls that reuse the array.
Runs last (file name) so that a failure here leaves every other test run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype):
    if a is None:
        return None
    return torch.from_numpy(np.ascontiguousarray(a).view(dtype)).cuda()


def _noalloc(genie, torch, table, qb, n_items=None, total_k=None):
    """Call genie_search_noalloc with every array in device memory (n_items /
    total_k: the host sizes passed, by default the batch's own)."""
    lib = genie.lib()
    t = dict(item_off=_dev(torch, qb.item_off, np.int64), dim=_dev(torch, qb.dim, np.int32),
             low=_dev(torch, qb.low, np.int32), up=_dev(torch, qb.up, np.int32),
             weight=_dev(torch, qb.weight, np.float32), weighted=_dev(torch, qb.weighted, np.uint8),
             k=_dev(torch, qb.k, np.int32), out_off=_dev(torch, qb.out_off, np.int64))
    n = qb.total_k
    ids = torch.zeros(n, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    sc = torch.zeros(n, dtype=torch.float32, device="cuda")
    s = genie._lib.GenieQueries()
    s.n_queries = qb.n_queries
    for f in ("item_off", "dim", "low", "up", "weight", "weighted", "k"):
        setattr(s, f, None if t[f] is None else t[f].data_ptr())
    s.uniform_k = qb.uniform_k
    rc = lib.genie_search_noalloc(table.handle, ctypes.byref(s), t["out_off"].data_ptr(),
                                  len(qb.dim) if n_items is None else n_items, n if total_k is None else total_k,
                                  ids.data_ptr(), cnt.data_ptr(), sc.data_ptr(), None)
    genie._check(rc)
    return (ids.cpu().numpy().view(np.uint32), cnt.cpu().numpy().view(np.uint32), sc.cpu().numpy())


def _qb(genie, b):
    return genie.QueryBatch(b["item_off"], b["dim"], b["low"], b["up"], b["k"], b.get("weight"), b.get("weighted"))


def test_noalloc_equals_search_on_consecutive_calls(genie):
    import torch
    from genie_gb300 import workloads
    values, mixed = workloads.config3(n=200_000, q=48)
    table = genie.Table.from_values(values)
    _, exact = workloads.config0(n=200, q=40, k=25, seed=9)      # exact items, uniform k
    for b in (mixed, exact, mixed):
        qb = _qb(genie, b) if b is mixed else genie.QueryBatch(b["item_off"], b["dim"], b["low"], b["up"], 25)
        want = genie.search(table, qb, scores=True)
        got = _noalloc(genie, torch, table, qb)
        for w, g_ in zip(want, got):
            assert np.array_equal(w, g_)


def test_noalloc_rejects_batches_beyond_its_fixed_workspace(genie):
    import torch
    table = genie.Table.from_values(np.zeros((10, 2), np.int32))
    q = 2000
    qb = genie.QueryBatch(np.arange(q + 1), np.zeros(q), np.zeros(q), np.zeros(q), 1)
    with pytest.raises(genie.cpu_runtime_error, match="at most 1024 queries"):
        _noalloc(genie, torch, table, qb)


def test_noalloc_takes_no_device_memory(genie):
    """After a first call, further calls leave the device's free memory as it
    was: the entry point allocates nothing."""
    import torch
    from genie_gb300 import workloads
    values, b = workloads.config3(n=100_000, q=32)
    table = genie.Table.from_values(values)
    qb = _qb(genie, b)
    want = _noalloc(genie, torch, table, qb)          # first call: symbol lookup and kernel set-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        got = _noalloc(genie, torch, table, qb)
        for w, g_ in zip(want, got):
            assert np.array_equal(w, g_)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_sizes_that_disagree_with_the_device_arrays(genie):
    """item_off[n_queries] above the n_items passed, or result slots past
    total_k, are refused on the device before anything is written; the next
    consistent call is still exact."""
    import torch
    from genie_gb300 import workloads
    values, b = workloads.config3(n=50_000, q=16)
    table = genie.Table.from_values(values)
    qb = _qb(genie, b)
    with pytest.raises(genie.cpu_runtime_error, match="outside the batch's arrays"):
        _noalloc(genie, torch, table, qb, n_items=len(qb.dim) - 1)
    with pytest.raises(genie.cpu_runtime_error, match="outside the batch's arrays"):
        _noalloc(genie, torch, table, qb, total_k=qb.total_k - 1)
    want = genie.search(table, qb, scores=True)
    for w, g_ in zip(want, _noalloc(genie, torch, table, qb)):
        assert np.array_equal(w, g_)


def test_noalloc_rejects_range_items_beyond_its_unit_capacity(genie):
    """One range item over 300,000 distinct values covers 300,000 lists, more
    than the 262,144 list units of the fixed workspace: the call is refused,
    and the next call is exact."""
    import torch
    n = 300_000
    table = genie.Table.from_values(np.arange(n, dtype=np.int32).reshape(n, 1))
    wide = genie.QueryBatch(np.array([0, 1]), np.array([0]), np.array([0]), np.array([n - 1]), 5)
    with pytest.raises(genie.cpu_runtime_error, match="unit capacity"):
        _noalloc(genie, torch, table, wide)
    ok = genie.QueryBatch(np.array([0, 2]), np.array([0, 0]), np.array([7, 100]), np.array([9, 100]), 5)
    want = genie.search(table, ok, scores=True)
    for w, g_ in zip(want, _noalloc(genie, torch, table, ok)):
        assert np.array_equal(w, g_)
