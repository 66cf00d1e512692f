#!/usr/bin/env python
"""Benchmark of GB300-native GENIE match-count top-k search.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload config0|config1|config2|config3]

A step is one batch of the batched-uneven workload (the default, config3):
10,000,000 objects x 128 dims of half-normal byte values (30% zeros), 16,384
queries of 8-128 items on distinct dims with range half-width r in {0,1,2,4},
half of them weighted with FP32 weights U[0.5,2], k in {10,100}, searched to
exact top-k.  Prints one JSON line:

  value      queries/s with the batch resident in HBM: the captured CUDA graph
             (device-side query compile + persistent match kernels + top-k),
             CUDA events on the launching stream, L2 flushed before every step
  e2e        queries/s through the public batch API from host buffers: every
             step uploads its queries and downloads its ids/counts; two
             batches in turn (genie_batch_submit / genie_batch_collect);
             e2e.sequential_value is one genie_batch_run per step
  plain_e2e  the plain per-batch path (genie_search) on the same batch
  roofline   posting-list bytes touched per launch / the dominant kernel's
             event-timed duration, against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle on this host's cores over a prefix of the
             batch, and whether the GPU's ids, counts and scores equal it
             (weighted scores also within 1e-6 relative of an FP64 sum)
  legs       the default run adds the LSH-style workload (config1: 1,000,000
             x 240, 1,024 exact queries, k=100) with the same measurements,
             and the serving workload (config4: the config1, config3 and
             config2 indexes resident together at full size, Poisson
             arrivals, memory-budget admission, p50/p99 beside the plain
             per-batch path)

Under torchrun (N > 1) every rank searches its own replica of the index
(weak scaling; the path needs no data exchange between replicas) and the
slowest rank's time counts.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "queries/s and % HBM roofline at exact top-k; p50/p99 latency served vs plain"

WORKLOADS = {
    "config0": ("config0 plain small: 1,000 objects x 128 dims, uint8 half-normal values with 30% zeros; "
                "100 queries of 128 exact items from perturbed stored objects; k=10", 1000, 100),
    "config1": ("config1 LSH-style index: 1,000,000 objects x 240 dims, uint32 bucket ids uniform in "
                "[0,8192); 1,024 queries x 240 exact-match items (half derived from stored objects, 60% "
                "of items redrawn); k=100; exact top-k ids+counts", 1_000_000, 1024),
    "config2": ("config2 compressed: 10,000,000 objects x 32 dims, Zipf(1.1) over 65,536 terms; lists "
                "in 128-id segments, SERIAL_DELTA_COMP_BP32_VARINT; 4,096 queries x 32 Zipf items; k=32",
                10_000_000, 4096),
    "config3": ("config3 batched uneven: 10,000,000 objects x 128 dims uint8 half-normal (30% zeros); 16,384 "
                "queries of 8-128 items on distinct dims, ranges r in {0,1,2,4}, half weighted U[0.5,2], "
                "k in {10,100}; exact top-k ids+counts+scores", 10_000_000, 16384),
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="config3", choices=sorted(WORKLOADS),
                   help="config3 (default) is the headline; the others use the same line format")
    p.add_argument("--objects", type=int, default=0, help="objects (0: the workload's own size)")
    p.add_argument("--queries", type=int, default=0, help="queries per batch (0: the workload's own)")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--no-legs", action="store_true", help="skip the config1 and serving legs of the default run")
    p.add_argument("--no-serve", action="store_true", help="skip the serving (config 4) leg")
    p.add_argument("--serve-seconds", type=float, default=0.2, help="arrival window per offered rate")
    p.add_argument("--serve-budget", type=int, default=16 << 20,
                   help="memory budget (bytes of in-flight request state) of the serving leg")
    p.add_argument("--profile-batch", type=int, default=0,
                   help="only run the workload's batch this many times without a graph (for ncu), print its "
                        "per-kernel times and exit")
    p.add_argument("--tuning", default="",
                   help="fixed kernel shape, e.g. sparse_slots=53248,sparse_ctas_per_sm=1 (skips autotuning)")
    return p.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel, workload):
    """traffic_bytes_per_launch recorded in profiles/ for this kernel/workload
    (a capture of a smaller case states it scaled to the full launch)."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for name in sorted(os.listdir(pdir)):
        if not name.endswith((".md", ".txt")):
            continue
        with open(os.path.join(pdir, name)) as f:
            txt = f.read()
        if ("workload: " + workload) not in txt or ("kernel: " + kernel) not in txt:
            continue
        m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", txt)
        if m:
            return float(m.group(1))
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def count(self):
        return len(self.lines)

    def wait_samples(self, n, work, limit_s=5.0):
        """Run `work` (untimed launches of the same batch) until n samples exist."""
        t0 = time.time()
        while self.proc and self.count() < n and time.time() - t0 < limit_s:
            work()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local, dist


def max_over_ranks(x, dist, device_is_cuda):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if device_is_cuda else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gen_workload(name, workloads, objects=0, queries=0):
    """Seeded values and query batch of the workload (host only)."""
    desc, n0, q0 = WORKLOADS[name]
    n = objects or n0
    q = queries or q0
    values, batch = getattr(workloads, name)(n=n, q=q)
    return values, batch, desc, n


def make_table(g, name, values):
    return g.Table.compressed(values, 13, 128) if name == "config2" else g.Table.from_values(values)


def alg_bytes_of(name, table, batch, workloads):
    """Posting-list bytes the batch touches: 4 B per posting id in the clamped
    spans, or the encoded words x 4 of the covered segments (compressed)."""
    lay = table.layout()
    offs = lay["key_offsets"]
    if name == "config2":
        c = table.compressed_layout()
        offs = c["seg_word_off"][c["key_seg"]]
    return workloads.algorithmic_bytes(offs, lay["key_base"], lay["dim_min"], lay["dim_max"], batch)


def qbatch(g, b):
    return g.QueryBatch(b["item_off"], b["dim"], b["low"], b["up"], b["k"], b.get("weight"), b.get("weighted"))


def fp64_score_error(values, batch, ids, cnt, scores, out_off):
    """Largest relative difference between the GPU's weighted scores and an
    FP64 sum of the matched items' weights, over the weighted queries."""
    worst = 0.0
    wf = batch.get("weighted")
    if wf is None:
        return worst
    off = batch["item_off"]
    for q in np.nonzero(wf)[0]:
        a, z = off[q], off[q + 1]
        o, kq = int(out_off[q]), int(batch["k"][q])
        sel = cnt[o:o + kq] > 0
        if not sel.any():
            continue
        rid = ids[o:o + kq][sel].astype(np.int64)
        v = values[rid][:, batch["dim"][a:z]]
        hit = (v >= batch["low"][a:z]) & (v <= batch["up"][a:z])
        ref = (hit * batch["weight"][a:z].astype(np.float64)).sum(axis=1)
        err = np.abs(scores[o:o + kq][sel].astype(np.float64) - ref) / ref
        worst = max(worst, float(err.max()))
    return worst


def cpu_check(values, batch, name, ids_g, cnt_g, sc_g, cpu_seconds, workloads):
    """The oracle on this host's cores over the batch (or its first queries in
    growing samples when the whole batch would take longer than cpu_seconds),
    and its agreement with the GPU's results."""
    from oracle import oracle
    cores = os.cpu_count() or 1
    t_build = time.perf_counter()
    ox = oracle.Index(values)
    t_build = time.perf_counter() - t_build
    Q = len(batch["k"])
    sq = min(Q, 64)
    while True:
        sub = workloads.take_queries(batch, np.arange(sq))
        t0 = time.perf_counter()
        oid, ocnt, osc, ooff = ox.search(sub, n_threads=cores)
        dt = time.perf_counter() - t0
        if sq == Q or dt * 2 > cpu_seconds:
            break
        sq = min(Q, sq * 4)
    reps, t_cpu = 1, dt
    while sq == Q and t_cpu < cpu_seconds:
        t0 = time.perf_counter()
        ox.search(sub, n_threads=cores)
        t_cpu += time.perf_counter() - t0
        reps += 1
    nk = int(sub["k"].sum())
    out = {"value": sq * reps / t_cpu, "unit": "queries/s", "cores": cores, "kind": "port",
           "sample": "the first %d of the %d queries x %d repetitions (oracle index build %.1f s, untimed)"
                     % (sq, Q, reps, t_build),
           "matches_gpu": bool(np.array_equal(oid, ids_g[:nk]) and np.array_equal(ocnt, cnt_g[:nk])),
           "checked_queries": sq}
    if sc_g is not None:
        out["scores_match_gpu"] = bool(np.array_equal(osc, sc_g[:nk]))
        out["max_rel_err_vs_fp64"] = fp64_score_error(values, sub, ids_g[:nk], cnt_g[:nk], sc_g[:nk], ooff)
    return out


def measure(g, workloads, name, values, table, batch, desc, steps, warmup, stream, flush, dist, world,
            args, clocks_device=None, cpu=True, rotate=None):
    """Every measurement of one workload: graph value, per-kernel roofline,
    e2e (pipelined and sequential), plain per-batch path, CPU oracle."""
    import torch
    alg = alg_bytes_of(name, table, batch, workloads)
    qb = qbatch(g, batch)
    n_items = int(batch["item_off"][-1])
    Q = qb.n_queries
    max_k = int(np.max(batch["k"]))
    weighted = batch.get("weighted") is not None and bool(np.any(batch["weighted"]))

    bt = g.Batch(table, Q, n_items, max_k, use_graph=True)
    if args.tuning:
        bt.set_tuning(**{kv.split("=")[0]: int(kv.split("=")[1]) for kv in args.tuning.split(",")})
        tuning = bt.tuning()
    elif args.no_autotune:
        tuning = bt.tuning()
    else:       # tune on (at most) the first 1,024 queries
        sq = min(Q, 1024)
        tuning = bt.autotune(qbatch(g, workloads.take_queries(batch, np.arange(sq))))
    bt.stage(qb)

    # ---- value: device-resident batch, graph launches, L2 flushed per step
    for _ in range(warmup):
        flush.zero_()
        bt.launch(stream.cuda_stream)
    torch.cuda.synchronize()

    def load():     # untimed steps of the same batch, so that clock samples see the GPU under load
        for _ in range(2):
            flush.zero_()
            bt.launch(stream.cuda_stream)
        torch.cuda.synchronize()

    clocks = None
    if clocks_device is not None:
        clocks = Clocks(clocks_device)
        clocks.start()
        clocks.wait_samples(2, load)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    n0 = clocks.count() if clocks else 0
    for s, e in evs:
        flush.zero_()
        s.record(stream)
        bt.launch(stream.cuda_stream)
        e.record(stream)
    torch.cuda.synchronize()
    step_ms = [s.elapsed_time(e) for s, e in evs]
    clock_info = None
    if clocks:
        in_region = clocks.count() - n0
        clocks.wait_samples(clocks.count() + 2, load)
        clock_info = clocks.stop()
        clock_info["window"] = ("200 ms samples: %d inside the timed region, the rest over untimed steps of the "
                                "same batch right before and after it" % in_region)
    total_ms = max_over_ranks(sum(step_ms), dist, True)
    value = world * Q * steps / (total_ms / 1e3)
    kernels_per_step = bt.last_stats()[0]
    want_scores = weighted
    if want_scores:
        ids_graph, cnt_graph, sc_graph = bt.fetch(scores=True)
    else:
        ids_graph, cnt_graph = bt.fetch()
        sc_graph = None
    ms_step = total_ms / steps
    # the secondary legs take about 15 s each at most
    aux = max(3, min(steps, int(15000.0 / max(ms_step, 1e-3))))

    # ---- roofline: per-kernel events (direct launches, same tuning and flushing)
    bp = g.Batch(table, Q, n_items, max_k, use_graph=False)
    bp.set_tuning(**{k: v for k, v in tuning.items()})
    bp.stage(qb)
    stage_tot = np.zeros(4)
    for i in range(1 + aux):
        flush.zero_()
        bp.launch(stream.cuda_stream)
        ms = bp.stage_ms()
        if i >= 1:
            stage_tot += ms
    del bp
    names = ["k_plan", "k_bitmap", "k_sparse", "k_dense"]
    # the match kernels that carry the batch (>= 15% of the match time); when
    # several share it, their posting bytes are counted over their summed time
    match_ms = stage_tot[1:]
    busy = [i + 1 for i in range(len(match_ms)) if match_ms[i] >= 0.15 * match_ms.sum()]
    dom = int(np.argmax(stage_tot[1:]) + 1)
    dom_ms = float(sum(stage_tot[i] for i in busy)) / aux
    peak, peak_kind = peaks()
    achieved = alg / (dom_ms / 1e3) / 1e9
    traffic = ncu_traffic(names[dom], name) if len(busy) == 1 else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": "+".join(names[i] for i in busy), "kernel_ms": dom_ms,
                "algorithmic_bytes_per_launch": alg, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else peak_kind, "launches_timed": aux,
                "stage_ms": {n: float(v / aux) for n, v in zip(names, stage_tot)}}

    # ---- e2e through the public API from host buffers.  Sequential: one
    # genie_batch_run per step (L2 flushed before each, outside the timing).
    bt.run(qb)
    e2e_times = []
    for _ in range(aux):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bt.run(qb)
        e2e_times.append(time.perf_counter() - t0)
    e2e_seq = world * Q * aux / max_over_ranks(sum(e2e_times), dist, True)
    # Pipelined (the e2e number): two batches in turn through genie_batch_submit
    # / genie_batch_collect, so that one batch's host-side staging overlaps the
    # other's device work.  Every step still uploads its queries from host
    # memory and downloads its results.
    rot = [qb] + [qbatch(g, r) for r in (rotate or [])]
    bt2 = g.Batch(table, Q, n_items, max_k, use_graph=True)
    bt2.set_tuning(**{k: v for k, v in tuning.items()})
    pair = (bt, bt2)

    def pipeline(n):
        pend = []
        out = None
        for i in range(n):
            b = pair[i % 2]
            if len(pend) == 2:
                pend.pop(0).collect()
            b.submit(rot[i % len(rot)], scores=want_scores)
            pend.append(b)
        for b in pend:
            out = b.collect()
        return out

    pipeline(min(4, max(2, warmup)))
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    pipeline(steps)
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, True)
    e2e = world * Q * steps / e2e_s
    bt.submit(qb, scores=want_scores)
    got = bt.collect()
    pipelined_same = bool(np.array_equal(got[0], ids_graph) and np.array_equal(got[1], cnt_graph))
    del bt2
    exact = batch.get("weight") is None and np.array_equal(batch["low"], batch["up"])
    h2d = (Q + 1) * 8 + n_items * (8 if exact else 12) + Q * 4
    if batch.get("weight") is not None:
        h2d += n_items * 4 + Q
    d2h = qb.total_k * (12 if want_scores else 8) + 4

    # ---- plain per-batch path (genie_search) for the batched/plain ratio
    g.search(table, qb)
    plain_times = []
    for _ in range(aux):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pid, pcnt = g.search(table, qb)
        plain_times.append(time.perf_counter() - t0)
    plain = world * Q * aux / max_over_ranks(sum(plain_times), dist, True)
    same = bool(np.array_equal(pid, ids_graph) and np.array_equal(pcnt, cnt_graph))
    del bt

    out = {
        "workload": desc, "value": value, "unit": "queries/s", "ms_per_step": ms_step, "steps": steps,
        "n_objects": int(values.shape[0]), "n_dims": int(values.shape[1]), "n_queries": Q,
        "k": max_k if int(np.min(batch["k"])) == max_k else "per query (%d..%d)" % (int(np.min(batch["k"])), max_k),
        "tuning": tuning,
        "e2e": {"value": e2e, "unit": "queries/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "genie_batch_submit / genie_batch_collect, two batches in turn over %d query batch(es)"
                        % len(rot), "same_results": pipelined_same, "sequential_value": e2e_seq,
                "sequential_steps": aux},
        "plain_e2e": {"value": plain, "unit": "queries/s", "path": "genie_search (per-call upload and launch)",
                      "batched_over_plain": e2e / plain, "same_results": same, "steps": aux},
        "roofline": roofline,
        "gpu_launches": kernels_per_step * steps,
        "clocks": clock_info,
        "results": (ids_graph, cnt_graph, sc_graph),
    }
    if cpu:
        out["cpu_baseline"] = cpu_check(values, batch, name, ids_graph, cnt_graph, sc_graph, args.cpu_seconds,
                                        workloads)
    return out


def serve_leg(g, workloads, tables, pools, args):
    """Config 4 (serving): the config1, config3 and config2 indexes (the last
    compressed with SERIAL_DELTA_COMP_BP32_VARINT in 128-id segments) resident
    together at full size; open-loop Poisson arrivals at 10k, 50k and 200k
    requests/s drawn 2:1:1 from the config3 : config1 : config2 query
    generators; one query per request; admission by a memory budget over the
    requests' device state.  Latency = answer ready - arrival.  Beside it,
    the same request mix through the plain per-batch path (genie_search, 256
    queries per call)."""
    srv = g.Server(max_queries=256, max_items=256 * 240, max_k=100, slots_per_index=2, window_us=100,
                   memory_budget=args.serve_budget)
    ids = [srv.add_index(t) for t in tables]
    srv.start()
    rates = {}
    mixes = {}
    for rate in (10_000, 50_000, 200_000):
        n = max(64, int(rate * args.serve_seconds))
        rng = np.random.default_rng(rate)
        which = rng.choice(np.array([1, 1, 0, 2]), size=n)         # 2:1:1 config3 : config1 : config2
        start = srv.now_ns() + 200_000_000 + n * 3_000             # after every submission below
        arrivals = g.poisson_arrivals(rate, n, seed=rate + 1, start_ns=start)
        srv.reset_stats()
        subs, mix = [], []
        for j in range(3):
            sel = np.nonzero(which == j)[0]
            if sel.size == 0:
                continue
            qs = rng.integers(0, pools[j]["k"].shape[0], sel.size)
            sub = workloads.take_queries(pools[j], qs)
            qb = qbatch(g, sub)
            first = srv.submit(ids[j], qb, arrivals[sel])
            subs.append((first, qb.k_array))
            mix.append((j, sub))
        srv.drain()
        st = srv.stats()
        for first, ks in subs:
            for i, k in enumerate(ks):
                srv.wait(first + i, int(k))
        rates[str(rate)] = {"offered_qps": rate, "requests": n, "sustained_qps": st["throughput_qps"],
                            "p50_us": st["p50_us"], "p99_us": st["p99_us"], "max_us": st["max_us"],
                            "mean_batch": st["mean_batch"], "held_by_budget": st["held"],
                            "peak_in_flight_bytes": st["peak_in_flight_bytes"]}
        mixes[rate] = mix
    srv.close()
    # each rate's request mix through the plain per-batch path
    for rate, mix in mixes.items():
        t0 = time.perf_counter()
        n_plain = 0
        for j, sub in mix:
            Qj = sub["k"].shape[0]
            for q0 in range(0, Qj, 256):
                part = workloads.take_queries(sub, np.arange(q0, min(Qj, q0 + 256)))
                qb = qbatch(g, part)
                g.search(tables[j], qb)
                n_plain += qb.n_queries
        plain_qps = n_plain / (time.perf_counter() - t0)
        r = rates[str(rate)]
        r["plain_per_batch_qps"] = plain_qps
        r["served_over_plain"] = r["sustained_qps"] / plain_qps
    return {"indexes": "config1 %d x 240; config3 %d x 128; config2 %d x 32 compressed" % (
                tables[0].i_size(), tables[1].i_size(), tables[2].i_size()),
            "mix": "2:1:1 config3 : config1 : config2, one query per request, Poisson arrivals, %.2f s of "
                   "arrivals per rate" % args.serve_seconds,
            "memory_budget_bytes": args.serve_budget,
            "rates": rates}


def run_reference(args, world, rank):
    """The reference's own CPU implementation of the path is its CPU
    match-count oracle (test/test_compression_query.cu:127-284); here the
    oracle restatement runs on all host threads over bounded samples."""
    if rank != 0:
        return
    from genie_gb300 import workloads
    from oracle import oracle
    values, batch, desc, _ = gen_workload(args.workload, workloads, args.objects, args.queries)
    ox = oracle.Index(values)
    cores = os.cpu_count() or 1
    # a sample of the batch that takes about a second per step
    Q = len(batch["k"])
    sample_q = min(Q, 16)
    while True:
        sub = workloads.take_queries(batch, np.arange(sample_q))
        t0 = time.perf_counter()
        ox.search(sub, n_threads=cores)
        dt = time.perf_counter() - t0
        if sample_q == Q or dt > 0.5:
            break
        sample_q = min(Q, sample_q * 2)
    for _ in range(max(0, args.warmup - 1)):
        ox.search(sub, n_threads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ox.search(sub, n_threads=cores)
    dt = time.perf_counter() - t0
    qps = sample_q * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": desc, "step": "%d-query sample of the batch" % sample_q},
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": cores, "kind": "port",
                         "sample": "%d queries of the %s batch per step, %d steps" % (sample_q, args.workload,
                                                                                     args.steps)},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    args = parse()
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        if dist is not None:
            dist.destroy_process_group()
        return
    import torch
    import genie_gb300 as g
    from genie_gb300 import build, workloads
    build.build()
    torch.cuda.set_device(local)
    g._check(g.lib().genie_init(local))

    values, batch, desc, n = gen_workload(args.workload, workloads, args.objects, args.queries)
    table = make_table(g, args.workload, values)
    if args.profile_batch:
        qb = qbatch(g, batch)
        bp = g.Batch(table, qb.n_queries, int(batch["item_off"][-1]), int(np.max(batch["k"])), use_graph=False)
        if args.tuning:
            bp.set_tuning(**{kv.split("=")[0]: int(kv.split("=")[1]) for kv in args.tuning.split(",")})
        bp.stage(qb)
        for _ in range(args.profile_batch):
            bp.launch()
            bp.fetch()
        print(json.dumps({"profile_batch": args.profile_batch, "workload": args.workload,
                          "stage_ms": [round(float(x), 4) for x in bp.stage_ms()]}))
        return

    # one non-default stream carries the L2 flushes, the events and the graph
    # launches (a null handle would select the batch's own stream instead)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")     # > 3x the 129 MB L2

    head = measure(g, workloads, args.workload, values, table, batch, desc, args.steps, args.warmup, stream,
                   flush, dist, world, args, clocks_device=local, cpu=(rank == 0))
    legs = {}
    default_run = args.workload == "config3" and not args.objects and not args.queries and not args.no_legs
    if default_run and rank == 0:
        v1, b1, d1, _ = gen_workload("config1", workloads)
        t1 = make_table(g, "config1", v1)
        rot = [workloads.config1_queries(v1, 1024, 100, seed=7000 + j) for j in range(3)]
        leg1 = measure(g, workloads, "config1", v1, t1, b1, d1, 20, 5, stream, flush, None, 1, args, cpu=True,
                       rotate=rot)
        leg1.pop("results")
        leg1.pop("clocks")
        legs["config1"] = leg1
        if not args.no_serve:
            v2, b2, _, _ = gen_workload("config2", workloads)
            t2 = make_table(g, "config2", v2)
            del v2
            legs["serving"] = serve_leg(g, workloads, [t1, table, t2], [b1, batch, b2], args)
    head.pop("results")

    if rank == 0:
        line = {
            "metric": METRIC, "value": head["value"], "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded generator with the %s shapes and distributions)" % args.workload,
            "config": {"workload": desc, "n_objects": head["n_objects"], "n_dims": head["n_dims"],
                       "n_queries": head["n_queries"], "k": head["k"],
                       "l2": "flushed by a 512 MiB device write before every timed step (the batch's posting "
                             "lists are also far larger than L2)",
                       "tuning": head["tuning"],
                       "parallelism": "replica per GPU" if world > 1 else "single GPU"},
            "e2e": head["e2e"],
            "plain_e2e": head["plain_e2e"],
            "roofline": head["roofline"],
            "cpu_baseline": head.get("cpu_baseline"),
            "clocks": head["clocks"],
            "gpu_launches": head["gpu_launches"],
            "legs": legs or None,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
