"""bench.py -- H2H build seconds and batched query throughput on GB300.

Workload (one GPU): the synthetic road graph with the size of DIMACS NY
(264,346 vertices, ~733,846 arcs, jittered grid on a 1:1.3 box plus a sparse
highway layer, int32 Euclidean weights), latitude/longitude partition of
height 10, ChangeToGlobalHeight 2, GPU contraction + GPU L4 labels.  A step is
one batch of 2*10^6 query pairs (10^6 uniform + 10^6 local, t within 20 hops
of s) answered in UsingLCA mode on the device-resident index.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N>1 runs under torchrun: every rank builds its own replica of the index and
answers its own batch (queries are independent: weak scaling, no collective
on the data path); the timed region is bracketed by barriers and the slowest
rank's time is reported.  `--impl reference` times the reference's CPU
algorithm (the oracle restatement of makeH2HLabel_noHub_multiThred and the
H2HDistancQuery_UsingLCA_noHub thread loop) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "gpu-h2h_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "H2H build s + queries/s on 1 GB300 vs plain GPU path; query p50/p99 latency"
WORKLOAD = dict(name="cfg1", n=264346, target_arcs=733846, aspect_milli=1300, jitter_milli=300, diag_permille=50,
                hw_tiers=1, hw_permille10=50, hw_k=3, hw_scale_milli=400, partition_height=10, seed=1)
H, C = 10, 2
Q_UNIFORM, Q_LOCAL, LOCAL_HOPS = 1_000_000, 1_000_000, 20


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def gen_graph(root: str):
    import gpuh2h
    kw = {k: v for k, v in WORKLOAD.items() if k != "name"}
    kw.update(cols=0, drop_permille=0)
    arcs = gpuh2h.generate_road(root, WORKLOAD["name"], **kw)
    return gpuh2h.files_for(root, WORKLOAD["name"]), arcs


def batched_build(threads: int, count: int) -> dict:
    """64 road graphs (log-uniform 2,000-200,000 vertices, partition height
    ceil(log2(n/256)), C = 2), built once as sequential single-graph builds
    (h2h_contract + h2h_build_labels per graph) and once as one batch
    (h2h_batch_build), then rebuilt from the device state after a weight
    update (h2h_batch_rebuild: one CUDA graph replay) with the default and the
    autotuned fill tile shapes.  Parity: every graph's answers to 10^4 seeded
    pairs, max label and label count equal its sequential build's."""
    import torch

    import gpuh2h
    root = tempfile.mkdtemp(prefix="h2h_batch_")
    params = gpuh2h.road_batch_params(count, 2000, 200000, seed=7)
    specs = []
    for i, p in enumerate(params):
        name = "g%02d" % i
        gpuh2h.generate_road(root, name, **p)
        specs.append((gpuh2h.files_for(root, name), p["partition_height"]))
    load = lambda: [gpuh2h.Graph("g", H, 2, threads, 1, files=f) for f, H in specs]
    seq = load()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for g in seq:
        g.contraction_noHub(1)
        g.constructLabel_noHub(2, 1, gpuh2h.LABEL_L4)
    seq_s = time.perf_counter() - t0
    bat = load()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = gpuh2h.Batch(bat, threads)
    batch_s = time.perf_counter() - t0
    cold = b.info()

    def check():
        for i, (gs, gb) in enumerate(zip(seq, bat)):
            n = gs.info()["n"]
            x, y = gpuh2h.uniform_pairs(n, 10_000, 100 + i)
            assert np.array_equal(gs.query(x, y), gb.query(x, y)), "batch graph %d answers differ" % i
            a, c = gs.info(), gb.info()
            assert a["max_label"] == c["max_label"] and a["label_size"] == c["label_size"]
    check()

    def rebuilds(k=5):
        ts = []
        for _ in range(k):
            b.rebuild()
            ts.append(b.info()["t_rebuild_us"] / 1e6)
        return statistics.median(ts)
    b.rebuild()  # first call captures the CUDA graph
    reb_default = rebuilds()
    t0 = time.perf_counter()
    policy = b.tune(1)
    tune_s = time.perf_counter() - t0
    reb_tuned = rebuilds()
    check()
    # label construction alone: one forest fill against the per-graph fills
    # (our dataflow fill, and the reference's level-by-level mapping)
    plain_ms, plain_bad = 0.0, 0
    for gs in seq:
        ms, bad = gs.fill_labels_plain("pair")
        plain_ms += ms
        plain_bad += bad
    assert plain_bad == 0, "the plain fill mapping disagrees with the labels"
    single_fill_ms = sum(gs.info()["t_fill_gpu_us"] for gs in seq) / 1e3
    nv = sum(gs.info()["n"] for gs in seq)
    out = {"graphs": count, "vertices": nv, "label_entries": sum(gs.info()["label_size"] for gs in seq),
           "sequential_s": seq_s, "batched_s": batch_s, "speedup_cold": seq_s / batch_s,
           "batched_phases_ms": {k[2:-3]: cold[k] / 1e3 for k in cold if k.startswith("t_") and k.endswith("_us")
                                 and not k.startswith("t_rebuild")},
           "elim_launches": cold["elim_launches"], "fill_tiles": cold["fill_tiles"],
           "rebuild_s_default_tiles": reb_default, "rebuild_s_tuned_tiles": reb_tuned,
           "speedup_rebuild_vs_sequential": seq_s / reb_tuned, "tuned_policy": policy, "tune_s": tune_s,
           "label_construction": {
               "batched_fill_ms": cold["t_fill_us"] / 1e3, "sequential_dataflow_fills_ms": single_fill_ms,
               "sequential_plain_fills_ms": plain_ms,
               "speedup_vs_plain": plain_ms / (cold["t_fill_us"] / 1e3),
               "speedup_vs_sequential_dataflow": single_fill_ms / (cold["t_fill_us"] / 1e3),
               "plain": "the reference's mapping: one thread per (v,u) pair, one launch + sync per tree level"},
           "parity": "answers to 1e4 pairs per graph, max label and label count equal the sequential builds'"}
    b.close()
    for g in seq + bat:
        g.close()
    shutil.rmtree(root, ignore_errors=True)
    return out


SERVE_BIG = dict(name="road6m", n=6262104, target_arcs=15248146, aspect_milli=1500, jitter_milli=300,
                 diag_permille=50, hw_tiers=1, hw_permille10=50, hw_k=3, hw_scale_milli=400, partition_height=15,
                 seed=4, cols=0, drop_permille=0)


def run_serving(args) -> int:
    """Serving: the 6,262,104-vertex road graph (1:1.5 box, partition height
    15) resident with 8 road graphs of 50k-1M vertices in one continuous-
    batching server; Poisson request streams (1-10^5 pairs per request,
    log-uniform, random graph) at 10^3-10^5 requests/s, latency of 10^5-pair
    requests on the large graph, and closed-loop throughput against the HBM
    roofline of the query kernel."""
    import torch

    import gpuh2h
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    threads = max(1, os.cpu_count() or 1)
    root = tempfile.mkdtemp(prefix="h2h_serve_")
    specs = [(SERVE_BIG["name"], {k: v for k, v in SERVE_BIG.items() if k != "name"})]
    for i, p in enumerate(gpuh2h.road_batch_params(8, 50_000, 1_000_000, seed=23)):
        specs.append(("res%d" % i, p))
    graphs, build = [], []
    for name, p in specs:
        t0 = time.perf_counter()
        arcs = gpuh2h.generate_road(root, name, **p)
        t_gen = time.perf_counter() - t0
        g, bt = build_index(gpuh2h.files_for(root, name), threads, H=p["partition_height"], C=2)
        i = g.info()
        build.append({"graph": name, "vertices": i["n"], "arcs": arcs, "partition_height": p["partition_height"],
                      "build_s": bt, "gen_s": t_gen, "tree_height": i["tree_height"],
                      "label_entries": i["label_size"], "device_gb": i["device_bytes"] / 1e9,
                      "phases_ms": {k[2:-3]: i[k] / 1e3 for k in i if k.startswith("t_") and k.endswith("_us")}})
        log("built %s: %d vertices, %.1f s, %.1f GB" % (name, i["n"], bt, i["device_bytes"] / 1e9))
        graphs.append(g)
    nv = [g.info()["n"] for g in graphs]
    srv = gpuh2h.Server(slots=args.serve_slots, slot_pairs=1 << 17)
    gids = [srv.add(g) for g in graphs]
    # parity: server answers equal the direct batch API on every graph
    for k, g in enumerate(graphs):
        x, y = gpuh2h.uniform_pairs(nv[k], 50_000, 900 + k)
        out = np.zeros(len(x), np.int32)
        r = srv.submit(gids[k], x, y, out)
        srv.wait(r)
        srv.release(r)
        assert np.array_equal(out, g.query(x, y)), "server answers differ on graph %d" % k
    pct = lambda v, q: float(np.percentile(np.asarray(v), q))
    runs = {}
    # 10^5-pair requests on the large graph: alone, and four in flight
    for inflight in (1, 4):
        srv.reset_stats()
        r = srv.load([gids[0]], [nv[0]], rate=0, size_lo=100_000, size_hi=100_000, requests=300,
                     inflight=inflight, seed=31 + inflight)
        st = srv.stats()
        runs["big_1e5_inflight%d" % inflight] = {
            "requests": r["requests"], "p50_us": pct(r["latency_us"], 50), "p99_us": pct(r["latency_us"], 99),
            "queries_per_s": r["pairs"] / r["wall_s"], "kernel_us_per_batch": st["kernel_us"] / max(1, st["batches"])}
    # open-loop Poisson streams over all graphs
    for rate in (1e3, 1e4, 1e5):
        srv.reset_stats()
        r = srv.load(gids, nv, rate=rate, duration_s=args.serve_seconds, size_lo=1, size_hi=100_000, seed=int(rate))
        st = srv.stats()
        runs["poisson_%d" % int(rate)] = {
            "requests": r["requests"], "pairs": r["pairs"], "late_submissions": r["late"],
            "p50_us": pct(r["latency_us"], 50), "p99_us": pct(r["latency_us"], 99),
            "p99_us_1e5_pair_requests": pct(r["latency_us"][r["sizes"] >= 50_000], 99)
            if np.any(r["sizes"] >= 50_000) else None,
            "queries_per_s": r["pairs"] / r["wall_s"], "batches": st["batches"], "max_inflight": st["max_inflight"]}
    # saturation: closed loop on the large graph
    srv.reset_stats()
    r = srv.load([gids[0]], [nv[0]], rate=0, size_lo=100_000, size_hi=100_000, requests=600, inflight=16, seed=77)
    st = srv.stats()
    xs, ys = gpuh2h.uniform_pairs(nv[0], 200_000, 4242)
    b_q = algorithmic_bytes(graphs[0], xs, ys) / len(xs)
    try:
        peak = float(json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))["hbm_gbs"])
        peak_src = "measured"
    except Exception:
        peak, peak_src = 6800.0, "fallback"
    sat_q = r["pairs"] / r["wall_s"]
    kern_q = r["pairs"] / (st["kernel_us"] / 1e6)
    runs["saturation"] = {"requests": r["requests"], "queries_per_s": sat_q, "p50_us": pct(r["latency_us"], 50),
                          "p99_us": pct(r["latency_us"], 99), "algorithmic_bytes_per_query": b_q,
                          "served_frac_of_hbm": sat_q * b_q / 1e9 / peak,
                          "kernel_queries_per_s": kern_q, "kernel_frac_of_hbm": kern_q * b_q / 1e9 / peak,
                          "peak_gbs": peak, "peak_source": peak_src}
    line = {"metric": "served queries/s and p50/p99 latency (continuous batching, resident graphs)",
            "impl": "ours", "unit": "queries/s", "value": sat_q, "n_gpus": 1, "higher_is_better": True,
            "dtype": "int32", "data": "synthetic",
            "config": {"workload": "road6m: 6,262,104 vertices (1:1.5 box, partition height 15, C=2) + 8 resident "
                                   "road graphs of 50k-1M vertices; requests of 1-1e5 pairs (log-uniform) to "
                                   "random graphs", "slots": args.serve_slots, "slot_pairs": 1 << 17},
            "build": build, "runs": runs,
            "parity": "server answers to 5e4 pairs per graph equal h2h_query_batch_host"}
    print(json.dumps(line), flush=True)
    srv.close()
    for g in graphs:
        g.close()
    shutil.rmtree(root, ignore_errors=True)
    return 0


LARGE = dict(name="road3m", n=3598623, target_arcs=8778114, aspect_milli=2000, jitter_milli=300, diag_permille=50,
             hw_tiers=3, hw_permille10=50, hw_k=3, hw_scale_milli=400, weight_max=200000, partition_height=14,
             seed=3, cols=0, drop_permille=0)


def run_large(args) -> int:
    """One large graph: 3,598,623 vertices / ~8.78M arcs (1:2 box, three
    highway tiers, weights in [1, 2e5]), partition height 14: build phases,
    label memory, and steps of 1e7 queries (half uniform, half local <= 20
    hops), UsingLCA, inputs resident."""
    import torch

    import gpuh2h
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    threads = max(1, os.cpu_count() or 1)
    root = tempfile.mkdtemp(prefix="h2h_large_")
    p = {k: v for k, v in LARGE.items() if k != "name"}
    arcs = gpuh2h.generate_road(root, LARGE["name"], **p)
    g, bt = build_index(gpuh2h.files_for(root, LARGE["name"]), threads, H=LARGE["partition_height"], C=2)
    info = g.info()
    n = info["n"]
    x, y = gpuh2h.uniform_pairs(n, 5_000_000, 71)
    lx, ly = g.local_pairs(5_000_000, LOCAL_HOPS, 72)
    x, y = np.concatenate([x, lx]), np.concatenate([y, ly])
    xd, yd = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    od, od2 = torch.empty_like(xd), torch.empty_like(xd)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    nq = len(x)
    for _ in range(args.warmup):
        g.query_device(xd.data_ptr(), yd.data_ptr(), od.data_ptr(), nq, gpuh2h.QUERY_LCA, sp)
    g.query_device(xd.data_ptr(), yd.data_ptr(), od2.data_ptr(), nq, gpuh2h.QUERY_NOLCA, sp)
    torch.cuda.synchronize()
    assert torch.equal(od, od2), "UsingLCA and noLCA answers differ"
    steps = max(3, min(args.steps, 20))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda._sleep(40_000_000)
    e0.record(stream)
    for _ in range(steps):
        g.query_device(xd.data_ptr(), yd.data_ptr(), od.data_ptr(), nq, gpuh2h.QUERY_LCA, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1000.0
    q_s = steps * nq / t
    sample = np.random.default_rng(5).choice(nq, 200_000, replace=False)
    b_q = algorithmic_bytes(g, x[sample], y[sample]) / len(sample)
    try:
        peak = float(json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))["hbm_gbs"])
        peak_src = "measured"
    except Exception:
        peak, peak_src = 6800.0, "fallback"
    line = {"metric": "queries/s on one large graph (plus its build)", "impl": "ours", "value": q_s,
            "unit": "queries/s", "n_gpus": 1, "steps": steps, "higher_is_better": True, "dtype": "int32",
            "data": "synthetic",
            "config": {"workload": "road3m: %d vertices / %d arcs (1:2 box, 3 highway tiers, weights <= 2e5), "
                                   "partition height 14, C=2; step = 1e7 queries (5e6 uniform + 5e6 local <= 20 "
                                   "hops), UsingLCA" % (n, arcs)},
            "build_s": bt, "build_phases_ms": {k[2:-3]: info[k] / 1e3 for k in info if k.startswith("t_")
                                                 and k.endswith("_us")},
            "index": {"tree_height": info["tree_height"], "label_entries": info["label_size"],
                      "label_gb": info["label_size"] * 4 / 1e9, "device_gb": info["device_bytes"] / 1e9,
                      "max_label": info["max_label"]},
            "roofline": {"bound": "hbm", "algorithmic_bytes_per_query": b_q, "achieved": q_s * b_q / 1e9,
                         "peak": peak, "unit": "GB/s", "frac": q_s * b_q / 1e9 / peak, "peak_source": peak_src},
            "parity": "UsingLCA answers equal noLCA answers on all 1e7 pairs (both exact with L4 labels)"}
    print(json.dumps(line), flush=True)
    g.close()
    shutil.rmtree(root, ignore_errors=True)
    return 0


def query_pairs(g, n_vertices: int, seed: int):
    import gpuh2h
    x, y = gpuh2h.uniform_pairs(n_vertices, Q_UNIFORM, seed)
    lx, ly = g.local_pairs(Q_LOCAL, LOCAL_HOPS, seed + 1000)
    return np.concatenate([x, lx]), np.concatenate([y, ly])


def algorithmic_bytes(g, x, y) -> int:
    """Sum over queries of 84 + 12*|pos(LCA)| bytes (UsingLCA mode): pair ids 8,
    firstAppeare 8, RMQHash 16, RMQ_ID 8, depth 8, pos_hash 16, dis_hash 16,
    result 4, and per LCA position 4 (pos) + 8 (two label entries)."""
    _, depth, first = g.tree()
    rh, ri = g.rmq()
    ph = g.labels_pos_hash()
    fa, fb = first[x].astype(np.int64), first[y].astype(np.int64)
    lo, hi = np.minimum(fa, fb), np.maximum(fa, fb)
    k = np.floor(np.log2(hi - lo + 1)).astype(np.int64)
    i1 = ri[rh[lo] + k]
    i2 = ri[rh[hi - (1 << k) + 1] + k]
    lca = np.where(depth[i1] <= depth[i2], i1, i2)
    kq = ph[lca + 1] - ph[lca]
    same = x == y
    return int(np.where(same, 12, 84 + 12 * kq).sum())


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled while the timed region runs."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.p = None

    def start(self):
        """Start sampling and return once five samples are in (NVML start-up
        stays outside the timed region)."""
        import threading
        self.lines = []
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                       "-i", str(self.gpu), "-lms", "50"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
            return
        settled = threading.Event()

        def reader():
            for line in self.p.stdout:
                self.lines.append(line)
                if len(self.lines) >= 5:
                    settled.set()
            settled.set()
        self.t = threading.Thread(target=reader, daemon=True)
        self.t.start()
        settled.wait(timeout=20)

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.1)
        self.p.terminate()
        self.p.wait(timeout=10)
        self.t.join(timeout=10)
        out = "".join(self.lines)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [s.strip() for s in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(value: float, world: int) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_query_seed(rank: int) -> int:
    """Each replica answers its own batch: seeds differ per rank."""
    return 7 + rank


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def build_index(files, threads: int, H: int = H, C: int = C):
    import gpuh2h
    t0 = time.perf_counter()
    g = gpuh2h.Graph(WORKLOAD["name"], H, C, threads, 1, files=files)
    g.contraction_noHub(1)
    g.constructLabel_noHub(2, 1, gpuh2h.LABEL_L4)
    return g, time.perf_counter() - t0


def cpu_reference_run(files, x, y, threads: int, budget_s: float):
    """The reference's CPU path restated (oracle): build + threaded query loop."""
    from oracle import oracle
    t0 = time.perf_counter()
    o = oracle.OracleGraph(*files, H, C, threads).contract()
    t1 = time.perf_counter()
    o.build_labels(l4=True, threads=threads)
    t2 = time.perf_counter()
    done, q_time, reps = 0, 0.0, 0
    while q_time < budget_s and reps < 50:
        s = time.perf_counter()
        o.query_batch(x, y, lca=True, threads=threads)
        q_time += time.perf_counter() - s
        done += len(x)
        reps += 1
    return o, dict(contract_s=t1 - t0, labels_s=t2 - t1, query_s=q_time, queries=done, reps=reps)


def run_reference_arm(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    import gpuh2h
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory(prefix="h2h_bench_") as root:
        files, arcs = gen_graph(root)
        # pairs from the same generator as the GPU arm (host-only helpers)
        import ctypes
        L = gpuh2h.load_library()
        h = ctypes.c_void_p()
        gpuh2h._check(L.h2h_load_files(*[f.encode() for f in files], b"cfg1", H, C, threads, 1, ctypes.byref(h)))
        ux, uy = gpuh2h.uniform_pairs(WORKLOAD["n"], Q_UNIFORM, 7)
        lx, ly = np.empty(Q_LOCAL, np.int32), np.empty(Q_LOCAL, np.int32)
        gpuh2h._check(L.h2h_gen_local_pairs(h, Q_LOCAL, LOCAL_HOPS, 7 + 1000, gpuh2h._p(lx), gpuh2h._p(ly)))
        L.h2h_free(h)
        x, y = np.concatenate([ux, lx]), np.concatenate([uy, ly])
        from oracle import oracle
        t0 = time.perf_counter()
        o = oracle.OracleGraph(*files, H, C, threads).contract()
        t1 = time.perf_counter()
        o.build_labels(l4=True, threads=threads)
        t2 = time.perf_counter()
        for _ in range(args.warmup):
            o.query_batch(x, y, lca=True, threads=threads)
        times = []
        for _ in range(args.steps):
            s = time.perf_counter()
            o.query_batch(x, y, lca=True, threads=threads)
            times.append(time.perf_counter() - s)
    total = sum(times)
    value = args.steps * len(x) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": "cfg1 road graph 264,346 vertices / %d arcs, H=10, C=2, L4 labels, 2e6 queries/step "
                               "(1e6 uniform + 1e6 local)" % arcs, "parallelism": "host threads"},
        "build_s": t2 - t0, "build_phases_s": {"contract": t1 - t0, "labels": t2 - t1},
        "cpu_baseline": {"value": value, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": "%d steps x %d queries, UsingLCA, %d threads" % (args.steps, len(x), threads)},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--build-reps", type=int, default=3)
    ap.add_argument("--latency-batches", type=int, default=200)
    ap.add_argument("--cpu-budget", type=float, default=10.0, help="seconds of CPU query work for cpu_baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-node-fill", action="store_true",
                    help="also time the reference's node-per-thread fill mapping (about a minute)")
    ap.add_argument("--batch-graphs", type=int, default=64, help="graphs of the batched-build measurement (0: skip)")
    ap.add_argument("--serve", action="store_true", help="run the serving measurement instead")
    ap.add_argument("--large", action="store_true", help="run the 3.6M-vertex single-graph measurement instead")
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-seconds", type=float, default=2.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.serve:
        return run_serving(args)
    if args.large:
        return run_large(args)

    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import gpuh2h
    threads = max(1, (os.cpu_count() or 1) // max(1, world))
    root = tempfile.mkdtemp(prefix="h2h_bench_%d_" % rank)
    files, arcs = gen_graph(root)
    # ---- build (whole H2H construction from the loaded files), best-of and median
    build_times, phases = [], None
    g = None
    for r in range(max(1, args.build_reps)):
        if g is not None:
            g.close()
        torch.cuda.synchronize()
        g, bt = build_index(files, threads)
        build_times.append(bt)
    info = g.info()
    phases = {k[2:-3]: info[k] / 1e3 for k in info if k.startswith("t_") and k.endswith("_us")}
    x, y = query_pairs(g, info["n"], rank_query_seed(rank))
    nq = len(x)
    xd = torch.from_numpy(x).cuda()
    yd = torch.from_numpy(y).cuda()
    od = torch.empty_like(xd)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    for _ in range(args.warmup):
        g.query_device(xd.data_ptr(), yd.data_ptr(), od.data_ptr(), nq, gpuh2h.QUERY_LCA, sp)
    torch.cuda.synchronize()
    # parity spot check of this batch against the noLCA form (both exact with L4)
    od2 = torch.empty_like(xd)
    g.query_device(xd.data_ptr(), yd.data_ptr(), od2.data_ptr(), nq, gpuh2h.QUERY_NOLCA, sp)
    torch.cuda.synchronize()
    assert torch.equal(od, od2), "UsingLCA and noLCA answers differ"
    # ---- timed region: K steps, device-resident inputs
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # a 20 ms device sleep ahead of the first event: every step is enqueued
    # before the timed region starts, so a host stall cannot idle the GPU in it
    torch.cuda._sleep(40_000_000)
    e0.record(stream)
    for _ in range(args.steps):
        g.query_device(xd.data_ptr(), yd.data_ptr(), od.data_ptr(), nq, gpuh2h.QUERY_LCA, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop()
    t_local = e0.elapsed_time(e1) / 1000.0
    t_max = reduce_max(t_local, world)
    value = world * args.steps * nq / t_max
    kernel_s = t_local / args.steps
    # ---- roofline of the query kernel
    abytes = algorithmic_bytes(g, x, y)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        peak, peak_src = 6800.0, "fallback"
    achieved = abytes / kernel_s / 1e9
    traffic = None
    tf = os.path.join(REPO, "profiles", "query_traffic.json")
    if os.path.exists(tf):
        try:
            traffic = json.load(open(tf)).get("dram_bytes_per_query")
            traffic = traffic * nq if traffic is not None else None
        except Exception:
            traffic = None
    # ---- plain GPU mapping (one thread per query, the reference's kernel layout)
    for _ in range(3):
        g.query_device_plain(xd.data_ptr(), yd.data_ptr(), od2.data_ptr(), nq, gpuh2h.QUERY_LCA, sp)
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps_plain = max(3, min(args.steps, 50))
    p0.record(stream)
    for _ in range(reps_plain):
        g.query_device_plain(xd.data_ptr(), yd.data_ptr(), od2.data_ptr(), nq, gpuh2h.QUERY_LCA, sp)
    p1.record(stream)
    torch.cuda.synchronize()
    plain_value = reps_plain * nq / (p0.elapsed_time(p1) / 1000.0)
    assert torch.equal(od, od2)
    # ---- e2e through the public host-buffer API (pinned host buffers)
    xh = torch.from_numpy(x).pin_memory()
    yh = torch.from_numpy(y).pin_memory()
    oh = torch.empty(nq, dtype=torch.int32).pin_memory()
    for _ in range(3):
        g.query_host_ptr(xh.data_ptr(), yh.data_ptr(), oh.data_ptr(), nq, gpuh2h.QUERY_LCA)
    barrier(world)
    e2e_steps = max(3, min(args.steps, 50))
    s = time.perf_counter()
    for _ in range(e2e_steps):
        g.query_host_ptr(xh.data_ptr(), yh.data_ptr(), oh.data_ptr(), nq, gpuh2h.QUERY_LCA)
    e2e_local = time.perf_counter() - s
    e2e_t = reduce_max(e2e_local, world)
    e2e_value = world * e2e_steps * nq / e2e_t
    assert np.array_equal(oh.numpy(), od.cpu().numpy())
    # ---- latency of 10^5-query batches (device-only and through the host API)
    bq = 100_000
    lat_dev, lat_e2e = [], []
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.latency_batches)]
    for i, (a, b) in enumerate(ev):
        off = (i * bq) % (nq - bq)
        a.record(stream)
        g.query_device(xd.data_ptr() + 4 * off, yd.data_ptr() + 4 * off, od.data_ptr() + 4 * off, bq,
                       gpuh2h.QUERY_LCA, sp)
        b.record(stream)
    torch.cuda.synchronize()
    lat_dev = [a.elapsed_time(b) * 1000.0 for a, b in ev]
    for i in range(args.latency_batches):
        off = (i * bq) % (nq - bq)
        s = time.perf_counter()
        g.query_host_ptr(xh.data_ptr() + 4 * off, yh.data_ptr() + 4 * off, oh.data_ptr() + 4 * off, bq,
                         gpuh2h.QUERY_LCA)
        lat_e2e.append((time.perf_counter() - s) * 1e6)
    # ---- batched construction of many graphs (rank 0, N=1 only)
    batched = None
    if rank == 0 and world == 1 and args.batch_graphs > 0:
        batched = batched_build(threads, args.batch_graphs)
    # ---- CPU baseline (rank 0, N=1 only): the reference's CPU algorithm on host cores
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        _, cb = cpu_reference_run(files, x, y, cores, args.cpu_budget)
        cpu = {"value": cb["queries"] / cb["query_s"], "unit": "queries/s", "cores": cores, "kind": "port",
               "sample": "%d x %d queries (UsingLCA, L4 labels) over %d host threads; oracle build %.1f s "
                         "(contract %.1f s + labels %.1f s)" % (cb["reps"], nq, cores,
                                                                 cb["contract_s"] + cb["labels_s"], cb["contract_s"],
                                                                 cb["labels_s"]),
               "build_s": cb["contract_s"] + cb["labels_s"]}
    pct = lambda v, q: float(np.percentile(np.asarray(v), q))
    # L4 fill: own rows read+written, separator lists, one ancestor entry per update
    fill_s = info["t_fill_gpu_us"] / 1e6
    fill_bytes = 8 * info["label_size"] + 8 * info["pos_size"] + 4 * info["label_updates"]
    plain_fill_ms, plain_fill_bad = g.fill_labels_plain("pair")
    assert plain_fill_bad == 0, "the plain fill mapping disagrees with the labels"
    fill = {"kernel": "fill_flow_kernel", "updates": info["label_updates"], "seconds": fill_s,
            "plain_gpu_seconds": plain_fill_ms / 1e3,
            "plain_gpu": "the reference's mapping: one thread per (v,u) pair, one launch + sync per tree level",
            "updates_per_s": info["label_updates"] / fill_s if fill_s > 0 else None,
            "algorithmic_bytes": fill_bytes,
            "achieved_gbs": fill_bytes / fill_s / 1e9 if fill_s > 0 else None,
            "frac_of_hbm": fill_bytes / fill_s / 1e9 / peak if fill_s > 0 else None}
    if args.plain_node_fill:
        # the reference's parallelFine=1 mapping: a minute on this graph, so only on request
        node_fill_ms, node_fill_bad = g.fill_labels_plain("node")
        assert node_fill_bad == 0, "the node-per-thread fill mapping disagrees with the labels"
        fill.update({"plain_node_gpu_seconds": node_fill_ms / 1e3,
                     "plain_node_gpu": "the reference's parallelFine=1 mapping: one thread per node, one launch + "
                                       "sync per tree level"})
    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": "cfg1 road graph 264,346 vertices / %d arcs (jittered 1:1.3 grid + highway layer), "
                               "lat/long partition H=10, C=2, GPU contraction + GPU L4 labels; step = 2e6 queries "
                               "(1e6 uniform + 1e6 local <=20 hops), UsingLCA" % arcs,
                   "queries_per_step": nq, "l2": "index %.2f GB resident > L2 (no flush)" % (info["device_bytes"] / 1e9),
                   "parallelism": "replicas x%d (queries sharded by rank)" % world},
        "build_s": statistics.median(build_times), "build_s_min": min(build_times),
        "build_phases_ms": phases, "label_fill": fill,
        "index": {"tree_height": info["tree_height"], "label_entries": info["label_size"],
                  "device_bytes": info["device_bytes"], "max_label": info["max_label"]},
        "latency_us_1e5": {"device_p50": pct(lat_dev, 50), "device_p99": pct(lat_dev, 99),
                           "e2e_p50": pct(lat_e2e, 50), "e2e_p99": pct(lat_e2e, 99)},
        "plain_gpu": {"value": plain_value, "unit": "queries/s", "what": "one thread per query (reference mapping)"},
        "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": 8 * nq, "d2h_bytes_per_step": 4 * nq},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_src, "algorithmic_bytes_per_launch": abytes,
                     "kernel": "query_tile_kernel<LCA>"},
        "clocks": clocks,
        "batched_build": batched,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    g.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
