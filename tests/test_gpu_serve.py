"""Serving loop (genie_server_*): every request's answer in the mix equals the
answer of the same query searched alone, admission limits, statistics."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _slice(b, q0, q1):
    off = b["item_off"]
    a, z = off[q0], off[q1]
    out = dict(item_off=off[q0:q1 + 1] - a, dim=b["dim"][a:z], low=b["low"][a:z], up=b["up"][a:z],
               k=b["k"][q0:q1])
    if b.get("weight") is not None:
        out["weight"] = b["weight"][a:z]
        out["weighted"] = b["weighted"][q0:q1]
    return out


def _qb(genie, b):
    return genie.QueryBatch(b["item_off"], b["dim"], b["low"], b["up"], b["k"], b.get("weight"),
                            b.get("weighted"))


def test_mixed_requests_equal_solo_answers(genie):
    from genie_gb300 import workloads
    v1, b1 = workloads.config1(n=100_000, q=96, k=100)
    v3, b3 = workloads.config3(n=150_000, q=96)
    v2, b2 = workloads.config2(n=200_000, q=96, k=32)
    t1 = genie.Table.from_values(v1)
    t3 = genie.Table.from_values(v3)
    t2 = genie.Table.compressed(v2, 13, 128)
    srv = genie.Server(max_queries=32, max_items=32 * 240, max_k=100, slots_per_index=2, window_us=200)
    ids_ = [srv.add_index(t) for t in (t1, t3, t2)]
    srv.start()
    # interleaved Poisson arrivals over the three indexes (2:1:1 mix of config3 : config1 : config2)
    plan = [(1, b3, q) for q in range(96)] + [(0, b1, q) for q in range(48)] + [(2, b2, q) for q in range(48)]
    rng = np.random.default_rng(5)
    rng.shuffle(plan)
    t0 = srv.now_ns() + 2_000_000
    arrivals = genie.poisson_arrivals(50_000, len(plan), seed=6, start_ns=t0)
    tickets = []
    for (ix, b, q), at in zip(plan, arrivals):
        tickets.append(srv.submit(ids_[ix], _qb(genie, _slice(b, q, q + 1)), int(at)))
    tables = [t1, t3, t2]
    for (ix, b, q), tk in zip(plan, tickets):
        k = int(b["k"][q])
        ids, cnt, sc, lat = srv.wait(tk, k)
        solo = _qb(genie, _slice(b, q, q + 1))
        sid, scnt, ssc = genie.search(tables[ix], solo, scores=True)
        assert np.array_equal(ids, sid) and np.array_equal(cnt, scnt), (ix, q)
        assert np.array_equal(sc, ssc), (ix, q)
        assert lat > 0
    st = srv.stats()
    assert st["completed"] == len(plan) == st["submitted"]
    assert st["batches"] < len(plan)          # requests shared batches
    assert 0 < st["p50_us"] <= st["p99_us"] <= st["max_us"]
    srv.close()


def test_admission_limits(genie):
    from genie_gb300 import workloads
    v1, b1 = workloads.config1(n=50_000, q=4, k=10)
    t1 = genie.Table.from_values(v1)
    srv = genie.Server(max_queries=4, max_items=300, max_k=16, slots_per_index=1)
    a = srv.add_index(t1)
    srv.start()
    big_k = _slice(b1, 0, 1)
    big_k["k"] = np.array([32], np.uint32)
    with pytest.raises(genie.gpu_bad_alloc):
        srv.submit(a, _qb(genie, big_k))
    two = _slice(b1, 0, 2)               # 240 items each: fits one per batch, not two
    t = srv.submit(a, _qb(genie, two))
    r0 = srv.wait(t, 10)
    r1 = srv.wait(t + 1, 10)
    for q, r in ((0, r0), (1, r1)):
        sid, scnt = genie.search(t1, _qb(genie, _slice(b1, q, q + 1)))
        assert np.array_equal(r[0], sid) and np.array_equal(r[1], scnt)
    st = srv.stats()
    assert st["rejected"] == 1 and st["completed"] == 2 and st["batches"] == 2
    srv.close()


def test_memory_budget_holds_requests_back(genie):
    """A budget that fits about two requests' device state: admission holds
    the rest until memory frees up, the in-flight peak never passes the
    budget, and every answer equals the same query searched alone."""
    from genie_gb300 import workloads
    v3, b3 = workloads.config3(n=120_000, q=24)
    t3 = genie.Table.from_values(v3)
    budget = 130_000                              # about two requests of k=100
    srv = genie.Server(max_queries=16, max_items=16 * 128, max_k=100, slots_per_index=2, window_us=0,
                       memory_budget=budget)
    a = srv.add_index(t3)
    srv.start()
    first = srv.submit(a, _qb(genie, b3))          # all 24 arrive at once
    for q in range(24):
        k = int(b3["k"][q])
        ids, cnt, sc, _ = srv.wait(first + q, k)
        sid, scnt, ssc = genie.search(t3, _qb(genie, _slice(b3, q, q + 1)), scores=True)
        assert np.array_equal(ids, sid) and np.array_equal(cnt, scnt) and np.array_equal(sc, ssc), q
    st = srv.stats()
    assert st["completed"] == 24
    assert st["held"] > 0
    assert 0 < st["peak_in_flight_bytes"] <= budget
    assert st["batches"] >= 4                     # the budget split the 24 requests into several batches
    srv.close()
