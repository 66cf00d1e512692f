#!/usr/bin/env python
"""Benchmark of GB300-native GENIE match-count top-k search.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one batch of the LSH-style workload (1,000,000 objects x 240 dims,
bucket ids uniform in [0, 8192), 1,024 queries of 240 exact items, half of
them derived from stored objects with 60% of items redrawn, k = 100) searched
to exact top-k.  Prints one JSON line:

  value      queries/s with the batch resident in HBM: the captured CUDA graph
             (device-side query compile + persistent match kernels + top-k),
             CUDA events on the launching stream, L2 flushed before every step
  e2e        queries/s through the public batch API from host buffers: every
             step uploads its queries and downloads its ids/counts; two
             batches in turn (genie_batch_submit / genie_batch_collect) over
             four query batches of the workload; e2e.sequential_value is one
             genie_batch_run per step
  roofline   posting-list bytes touched per launch / the dominant kernel's
             event-timed duration, against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle on this host's cores over the same batch

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
WORKLOAD = ("config1 LSH-style index: 1,000,000 objects x 240 dims, uint32 bucket ids uniform in "
            "[0,8192); 1,024 queries x 240 exact-match items (half derived from stored objects, 60% "
            "of items redrawn); k=100; exact top-k ids+counts")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="config1", choices=["config0", "config1", "config2", "config3"],
                   help="config1 (default) is the headline; the others use the same line format")
    p.add_argument("--objects", type=int, default=0, help="objects (0: the workload's own size)")
    p.add_argument("--queries", type=int, default=0, help="queries per batch (0: the workload's own)")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--no-serve", action="store_true", help="skip the serving (config 4) leg")
    p.add_argument("--serve-objects", type=int, default=1_000_000,
                   help="objects of the config2/config3 indexes resident beside config1 while serving")
    p.add_argument("--serve-seconds", type=float, default=0.2, help="arrival window per offered rate")
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
    """traffic_bytes_per_launch recorded in profiles/ for this kernel/workload."""
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
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
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


WORKLOADS = {
    "config0": ("config0 plain small: 1,000 objects x 128 dims, uint8 half-normal values with 30% zeros; "
                "100 queries of 128 exact items from perturbed stored objects; k=10", 1000, 100),
    "config1": (WORKLOAD, 1_000_000, 1024),
    "config2": ("config2 compressed: 10,000,000 objects x 32 dims, Zipf(1.1) over 65,536 terms; lists "
                "in 128-id segments, SERIAL_DELTA_COMP_BP32_VARINT; 4,096 queries x 32 Zipf items; k=32",
                10_000_000, 4096),
    "config3": ("config3 batched uneven: 10,000,000 objects x 128 dims uint8 half-normal; 16,384 queries "
                "of 8-128 items, ranges r in {0,1,2,4}, half weighted U[0.5,2], k in {10,100}",
                10_000_000, 16384),
}


def gen_workload(args, workloads):
    """Seeded values and query batch of the workload (host only)."""
    desc, n0, q0 = WORKLOADS[args.workload]
    n = args.objects or n0
    q = args.queries or q0
    gen = getattr(workloads, args.workload)
    values, batch = gen(n=n, q=q)
    return values, batch, desc, n


def load_workload(args, g, workloads):
    """Values, resident table, batch and algorithmic bytes of the workload."""
    values, batch, desc, n = gen_workload(args, workloads)
    if args.workload == "config2":
        table = g.Table.compressed(values, 13, 128)
    else:
        table = g.Table.from_values(values)
    lay = table.layout()
    offs = lay["key_offsets"]
    if args.workload == "config2":      # encoded words of the covered segments
        c = table.compressed_layout()
        offs = c["seg_word_off"][c["key_seg"]]
    alg = workloads.algorithmic_bytes(offs, lay["key_base"], lay["dim_min"], lay["dim_max"], batch)
    return dict(values=values, table=table, batch=batch, alg_bytes=alg, desc=desc, n=n, d=values.shape[1])


def serve_leg(g, workloads, t1, b1, args):
    """Config 4 (serving): the config1 index plus config3 and config2 indexes
    (the latter compressed with SERIAL_DELTA_COMP_BP32_VARINT in 128-id
    segments) resident together; open-loop Poisson arrivals at 10k, 50k and
    200k requests/s drawn 2:1:1 from the config3 : config1 : config2 query
    generators; one query per request.  Latency = answer ready - arrival.
    Beside it, the same request mix through the plain per-batch path
    (genie_search, 256 queries per call)."""
    import numpy as np
    v3, b3 = workloads.config3(n=args.serve_objects, q=4096)
    v2, b2 = workloads.config2(n=args.serve_objects, q=4096, k=32)
    t3 = g.Table.from_values(v3)
    t2 = g.Table.compressed(v2, 13, 128)
    del v3, v2
    srv = g.Server(max_queries=256, max_items=256 * 240, max_k=100, slots_per_index=2, window_us=100)
    tables = [t1, t3, t2]
    pools = [b1, b3, b2]
    ids = [srv.add_index(t) for t in tables]
    srv.start()
    rates = {}
    last_mix = None
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
            qb = g.QueryBatch(sub["item_off"], sub["dim"], sub["low"], sub["up"], sub["k"], sub["weight"],
                              sub["weighted"])
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
                            "mean_batch": st["mean_batch"]}
        last_mix = mix
    srv.close()
    # the same last mix through the plain per-batch path
    t0 = time.perf_counter()
    n_plain = 0
    for j, sub in last_mix:
        Qj = sub["k"].shape[0]
        for q0 in range(0, Qj, 256):
            part = workloads.take_queries(sub, np.arange(q0, min(Qj, q0 + 256)))
            qb = g.QueryBatch(part["item_off"], part["dim"], part["low"], part["up"], part["k"], part["weight"],
                              part["weighted"])
            g.search(tables[j], qb)
            n_plain += qb.n_queries
    plain_qps = n_plain / (time.perf_counter() - t0)
    return {"indexes": "config1 %d x 240; config3 %d x 128; config2 %d x 32 compressed" % (
                t1.i_size(), args.serve_objects, args.serve_objects),
            "mix": "2:1:1 config3 : config1 : config2, one query per request, Poisson arrivals",
            "rates": rates, "plain_per_batch_qps": plain_qps,
            "served_over_plain_at_200k": rates["200000"]["sustained_qps"] / plain_qps}


def run_reference(args, world, rank):
    """The reference's own CPU implementation of the path is its CPU
    match-count oracle (test/test_compression_query.cu:127-284); here the
    oracle restatement runs on all host threads over bounded samples."""
    if rank != 0:
        return
    from genie_gb300 import workloads
    from oracle import oracle
    values, batch, desc, _ = gen_workload(args, workloads)
    ox = oracle.Index(values)
    cores = os.cpu_count() or 1
    sample_q = min(256, len(batch["k"]))
    sub = workloads.take_queries(batch, np.arange(sample_q))
    for _ in range(max(1, args.warmup)):
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
    world, rank, local, dist = dist_setup(args.gpus)
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

    wl = load_workload(args, g, workloads)
    values, table, batch, alg_bytes = wl["values"], wl["table"], wl["batch"], wl["alg_bytes"]
    qb = g.QueryBatch(batch["item_off"], batch["dim"], batch["low"], batch["up"], batch["k"], batch.get("weight"),
                      batch.get("weighted"))
    n_items = int(batch["item_off"][-1])
    Q = qb.n_queries
    max_k = int(np.max(batch["k"]))
    if args.profile_batch:
        bp = g.Batch(table, Q, n_items, max_k, use_graph=False)
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
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")     # > 2x the 129 MB L2

    bt = g.Batch(table, Q, n_items, max_k, use_graph=True)
    if args.tuning:
        bt.set_tuning(**{kv.split("=")[0]: int(kv.split("=")[1]) for kv in args.tuning.split(",")})
        tuning = bt.tuning()
    elif args.no_autotune:
        tuning = bt.tuning()
    else:       # tune on (at most) the first 1,024 queries
        sq = min(Q, 1024)
        sub = workloads.take_queries(batch, np.arange(sq))
        tuning = bt.autotune(g.QueryBatch(sub["item_off"], sub["dim"], sub["low"], sub["up"], sub["k"],
                                          sub["weight"], sub["weighted"]))
    bt.stage(qb)

    # ---- value: device-resident batch, graph launches, L2 flushed per step
    for _ in range(args.warmup):
        flush.zero_()
        bt.launch(stream.cuda_stream)
    torch.cuda.synchronize()

    def load():     # untimed steps of the same batch, so that clock samples see the GPU under load
        for _ in range(4):
            flush.zero_()
            bt.launch(stream.cuda_stream)
        torch.cuda.synchronize()

    # the timed region lasts milliseconds, below nvidia-smi's 200 ms sampling
    # period: samples are taken over untimed steps right before and after it
    clocks = Clocks(local)
    clocks.start()
    clocks.wait_samples(2, load)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for s, e in evs:
        flush.zero_()
        s.record(stream)
        bt.launch(stream.cuda_stream)
        e.record(stream)
    torch.cuda.synchronize()
    step_ms = [s.elapsed_time(e) for s, e in evs]
    clocks.wait_samples(clocks.count() + 2, load)
    clock_info = clocks.stop()
    clock_info["window"] = "200 ms samples over untimed steps of the same batch around the timed region"
    total_ms = max_over_ranks(sum(step_ms), dist, True)
    value = world * Q * args.steps / (total_ms / 1e3)
    ids_graph, cnt_graph = bt.fetch()
    kernels_per_step = bt.last_stats()[0]

    # ---- roofline: per-kernel events (direct launches, same tuning and flushing)
    bp = g.Batch(table, Q, n_items, max_k, use_graph=False)
    bp.set_tuning(**{k: v for k, v in tuning.items()})
    bp.stage(qb)
    stage_tot = np.zeros(4)
    for i in range(args.warmup + args.steps):
        flush.zero_()
        bp.launch(stream.cuda_stream)
        ms = bp.stage_ms()
        if i >= args.warmup:
            stage_tot += ms
    names = ["k_plan", "k_bitmap", "k_sparse", "k_dense"]
    # the match kernels that carry the batch (>= 15% of the match time); when
    # several share it, their posting bytes are counted over their summed time
    match_ms = stage_tot[1:]
    busy = [i + 1 for i in range(len(match_ms)) if match_ms[i] >= 0.15 * match_ms.sum()]
    dom = int(np.argmax(stage_tot[1:]) + 1)
    dom_ms = float(sum(stage_tot[i] for i in busy)) / args.steps
    peak, peak_kind = peaks()
    achieved = alg_bytes / (dom_ms / 1e3) / 1e9
    traffic = ncu_traffic(names[dom], args.workload) if len(busy) == 1 else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": "+".join(names[i] for i in busy), "kernel_ms": dom_ms,
                "algorithmic_bytes_per_launch": alg_bytes, "peak_source": peak_kind,
                "stage_ms": {n: float(v / args.steps) for n, v in zip(names, stage_tot)}}

    # ---- e2e through the public API from host buffers.  Sequential: one
    # genie_batch_run per step (L2 flushed before each, outside the timing).
    for _ in range(max(1, args.warmup // 2)):
        bt.run(qb)
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bt.run(qb)
        e2e_times.append(time.perf_counter() - t0)
    e2e_seq = world * Q * args.steps / max_over_ranks(sum(e2e_times), dist, True)
    # Pipelined (the e2e number): two batches in turn through genie_batch_submit
    # / genie_batch_collect, so that one batch's host-side staging overlaps the
    # other's device work.  Every step still uploads its queries from host
    # memory and downloads its results.  The steps rotate over four query
    # batches of the workload whose posting lists together exceed L2.
    rot = [qb]
    if args.workload == "config1":
        for j in range(3):
            rb = workloads.config1_queries(values, Q, max_k, seed=7000 + j)
            rot.append(g.QueryBatch(rb["item_off"], rb["dim"], rb["low"], rb["up"], rb["k"]))
    bt2 = g.Batch(table, Q, n_items, max_k, use_graph=True)
    bt2.set_tuning(**{k: v for k, v in tuning.items()})
    pair = (bt, bt2)

    def pipeline(steps):
        pend = []
        for i in range(steps):
            b = pair[i % 2]
            if len(pend) == 2:
                pend.pop(0).collect()
            b.submit(rot[i % len(rot)])
            pend.append(b)
        out = None
        for b in pend:
            out = b.collect()
        return out

    pipeline(max(4, args.warmup))
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    pipeline(args.steps)
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, True)
    e2e = world * Q * args.steps / e2e_s
    # the rotation's first batch again, checked against the graph results
    bt.submit(qb)
    pid2, pcnt2 = bt.collect()
    pipelined_same = bool(np.array_equal(pid2, ids_graph) and np.array_equal(pcnt2, cnt_graph))
    h2d = (Q + 1) * 8 * 2 + n_items * 12 + Q + Q * 4 + 8
    d2h = qb.total_k * 8 + 4

    # ---- plain per-batch path (genie_search) for the batched/plain ratio
    for _ in range(max(1, args.warmup // 2)):
        g.search(table, qb)
    plain_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pid, pcnt = g.search(table, qb)
        plain_times.append(time.perf_counter() - t0)
    plain = world * Q * args.steps / max_over_ranks(sum(plain_times), dist, True)
    same = bool(np.array_equal(pid, ids_graph) and np.array_equal(pcnt, cnt_graph))

    # ---- CPU baseline: the oracle on this host's cores (rank 0), over the
    # whole batch repeated, or over its first queries in growing samples when
    # the whole batch would take longer than --cpu-seconds
    cpu = None
    if rank == 0:
        from oracle import oracle
        cores = os.cpu_count() or 1
        t_build = time.perf_counter()
        ox = oracle.Index(values)
        t_build = time.perf_counter() - t_build
        sq = min(Q, 64)
        while True:
            sub = workloads.take_queries(batch, np.arange(sq))
            t0 = time.perf_counter()
            oid, ocnt, _, _ = ox.search(sub, n_threads=cores)
            dt = time.perf_counter() - t0
            if sq == Q or dt * 2 > args.cpu_seconds:
                break
            sq = min(Q, sq * 4)
        reps, t_cpu = 1, dt
        while sq == Q and t_cpu < args.cpu_seconds:
            t0 = time.perf_counter()
            ox.search(sub, n_threads=cores)
            t_cpu += time.perf_counter() - t0
            reps += 1
        nk = int(sub["k"].sum())
        cpu = {"value": sq * reps / t_cpu, "unit": "queries/s", "cores": cores, "kind": "port",
               "sample": "the first %d of the %d queries x %d repetitions (oracle index build %.1f s, untimed)"
                         % (sq, Q, reps, t_build),
               "matches_gpu": bool(np.array_equal(oid, ids_graph[:nk]) and np.array_equal(ocnt, cnt_graph[:nk]))}

    serving = None
    if rank == 0 and not args.no_serve and args.workload == "config1":
        serving = serve_leg(g, workloads, table, batch, args)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded generator with the %s shapes and distributions)" % args.workload,
            "config": {"workload": wl["desc"], "n_objects": wl["n"], "n_dims": wl["d"], "n_queries": Q,
                       "k": max_k if int(np.min(batch["k"])) == max_k else "per query (%d..%d)" % (
                           int(np.min(batch["k"])), max_k),
                       "l2": "flushed by a 512 MiB device write before every timed step",
                       "tuning": tuning, "parallelism": "replica per GPU" if world > 1 else "single GPU"},
            "e2e": {"value": e2e, "unit": "queries/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": "genie_batch_submit / genie_batch_collect, two batches in turn over %d query batches"
                            % len(rot), "same_results": pipelined_same,
                    "sequential_value": e2e_seq},
            "plain_e2e": {"value": plain, "unit": "queries/s", "path": "genie_search (per-call upload and launch)",
                          "batched_over_plain": e2e / plain, "same_results": same},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "serving": serving,
            "clocks": clock_info,
            "gpu_launches": kernels_per_step * args.steps,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
