"""bench.py -- H2H build seconds and batched query throughput on GB300.

Default workload (one GPU): the 6,262,104-vertex synthetic road graph
(~15.25M arcs, the road generator over a 1:1.5 box with one highway tier,
int32 Euclidean weights), latitude/longitude partition of height 15,
ChangeToGlobalHeight 2, GPU contraction + GPU L4 labels (117 GB resident
index).  A step is one batch of 2*10^6 query pairs (10^6 uniform + 10^6 local,
t within 20 hops of s) answered in UsingLCA mode on the device-resident index.
The line also carries the build (phases), p50/p99 of 10^5-pair batches alone
and with four in flight through the continuous-batching server, e2e through
the host-buffer C ABI call, a Dijkstra check of sampled sources against every
target, and -- as extra keys -- the 264,346-vertex graph, the 64-graph
batched build and the reference's own GPU command line timed beside this
library's on the 4,096-vertex graph.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload road6m|cfg1|road3m] [--serve]

N>1 runs under torchrun: every rank builds its own replica of the index and
answers its own batch (queries are independent: weak scaling, no collective
on the data path); the timed region is bracketed by barriers and the slowest
rank's time is reported.  `--impl reference` times the reference's CPU
algorithm (the oracle restatement of the GPU-hybrid contraction,
makeH2HLabel_noHub_multiThred and the H2HDistancQuery_UsingLCA_noHub thread
loop) on the host cores; that process loads no GPU library.
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
import warnings

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "gpu-h2h_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "H2H build s + queries/s on 1 GB300 vs plain GPU path; query p50/p99 latency"

# Generator parameters of the named road graphs (seeded; the reference's
# Edge / ID / Cut formats).  C = ChangeToGlobalHeight.
WORKLOADS = {
    "road6m": dict(n=6262104, target_arcs=15248146, aspect_milli=1500, jitter_milli=300, diag_permille=50,
                   hw_tiers=1, hw_permille10=50, hw_k=3, hw_scale_milli=400, partition_height=15, seed=4, cols=0,
                   drop_permille=0),
    "cfg1": dict(n=264346, target_arcs=733846, aspect_milli=1300, jitter_milli=300, diag_permille=50, hw_tiers=1,
                 hw_permille10=50, hw_k=3, hw_scale_milli=400, partition_height=10, seed=1, cols=0, drop_permille=0),
    "road3m": dict(n=3598623, target_arcs=8778114, aspect_milli=2000, jitter_milli=300, diag_permille=50,
                   hw_tiers=3, hw_permille10=50, hw_k=3, hw_scale_milli=400, weight_max=200000,
                   partition_height=14, seed=3, cols=0, drop_permille=0),
}
DESCRIBE = {
    "road6m": "road6m: 6,262,104 vertices / %d arcs (jittered 1:1.5 grid + highway layer), lat/long partition "
              "H=15, C=2, GPU contraction + GPU L4 labels",
    "cfg1": "cfg1: 264,346 vertices / %d arcs (jittered 1:1.3 grid + highway layer), lat/long partition H=10, C=2, "
            "GPU contraction + GPU L4 labels",
    "road3m": "road3m: 3,598,623 vertices / %d arcs (1:2 box, 3 highway tiers, weights <= 2e5), lat/long partition "
              "H=14, C=2, GPU contraction + GPU L4 labels",
}
C_HEIGHT = 2
Q_UNIFORM, Q_LOCAL, LOCAL_HOPS = 1_000_000, 1_000_000, 20
# the CPU arms build this graph: the largest the reference's CPU algorithm
# finishes in a bounded run (its per-cell contraction restates the
# reference kernel's bubble sorts, cubic in a cell's size)
CPU_WORKLOAD = "cfg1"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def gen_graph(root: str, name: str):
    """Writes the named graph with the library's generator."""
    import gpuh2h
    arcs = gpuh2h.generate_road(root, name, **WORKLOADS[name])
    return gpuh2h.files_for(root, name), arcs


def build_index(files, threads: int, H: int, C: int = C_HEIGHT, name: str = "graph"):
    """G2H's load + contraction_noHub(1) + constructLabel_noHub(2, 1, L4)."""
    import gpuh2h
    t0 = time.perf_counter()
    g = gpuh2h.Graph(name, H, C, threads, 1, files=files)
    g.contraction_noHub(1)
    g.constructLabel_noHub(2, 1, gpuh2h.LABEL_L4)
    return g, time.perf_counter() - t0


def phases_ms(info: dict) -> dict:
    return {k[2:-3]: info[k] / 1e3 for k in info if k.startswith("t_") and k.endswith("_us")}


def query_pairs(g, n_vertices: int, seed: int, nu: int = Q_UNIFORM, nl: int = Q_LOCAL):
    import gpuh2h
    x, y = gpuh2h.uniform_pairs(n_vertices, nu, seed)
    lx, ly = g.local_pairs(nl, LOCAL_HOPS, seed + 1000)
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


def hbm_peak():
    try:
        return float(json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dijkstra_check(files, g, n: int, sources) -> dict:
    """Plain Dijkstra (scipy, parallel arcs reduced to their minimum, self
    loops dropped -- the loader's rules) from a few sources to every vertex,
    against the GPU answers of both query modes.  The Edge file is parsed
    here, independently of the library's loader."""
    import torch
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import dijkstra

    import gpuh2h
    t0 = time.perf_counter()
    raw = open(files[0], "rb").read()
    nl = raw.index(b"\n")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        v = np.fromstring(raw[nl + 1:].replace(b"a", b" ").decode(), dtype=np.int64, sep=" ")
    del raw
    v = v.reshape(-1, 3)
    u, t, w = v[:, 0] - 1, v[:, 1] - 1, v[:, 2]
    del v
    keep = u != t
    key = u[keep] * n + t[keep]
    w = w[keep]
    o = np.lexsort((w, key))
    key, w = key[o], w[o]
    first = np.ones(len(key), bool)
    first[1:] = key[1:] != key[:-1]
    key, w = key[first], w[first]
    m = csr_matrix((w.astype(np.float64), (key // n, key % n)), shape=(n, n))
    del key, w
    dist = dijkstra(m, directed=True, indices=np.asarray(sources, np.int64))
    t_dij = time.perf_counter() - t0
    yd = torch.arange(n, dtype=torch.int32, device="cuda")
    out = torch.empty_like(yd)
    sp = torch.cuda.current_stream().cuda_stream
    mism = {"lca": 0, "nolca": 0}
    for i, s in enumerate(sources):
        xd = torch.full((n,), int(s), dtype=torch.int32, device="cuda")
        ref = dist[i].astype(np.int64)
        for mode, k in ((gpuh2h.QUERY_LCA, "lca"), (gpuh2h.QUERY_NOLCA, "nolca")):
            g.query_device(xd.data_ptr(), yd.data_ptr(), out.data_ptr(), n, mode, sp)
            torch.cuda.synchronize()
            mism[k] += int((out.cpu().numpy().astype(np.int64) != ref).sum())
    return {"sources": [int(s) for s in sources], "targets_per_source": n, "mismatches_lca": mism["lca"],
            "mismatches_nolca": mism["nolca"], "dijkstra_s": t_dij,
            "what": "GPU answers (UsingLCA and noLCA) from each source to every vertex equal scipy Dijkstra on the "
                    "Edge file (parsed independently of the library)"}


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


def pct(v, q):
    return float(np.percentile(np.asarray(v), q))


def timed_queries(g, xd, yd, od, nq: int, steps: int, mode: int) -> float:
    """Device seconds of `steps` back-to-back batches (CUDA events on the
    launching stream; a device sleep ahead of the first event keeps host
    enqueue stalls out of the timed region)."""
    import torch
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    torch.cuda._sleep(40_000_000)
    e0.record(stream)
    for _ in range(steps):
        g.query_device(xd.data_ptr(), yd.data_ptr(), od.data_ptr(), nq, mode, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1000.0


def latency_runs(g, xd, yd, od, xh, yh, oh, nq: int, batches: int) -> dict:
    """p50/p99 of 10^5-pair batches: device only (events around the kernel)
    and through h2h_query_batch_host (host buffers, copies included)."""
    import torch

    import gpuh2h
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    bq = 100_000
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(batches)]
    for i, (a, b) in enumerate(ev):
        off = (i * bq) % (nq - bq)
        a.record(stream)
        g.query_device(xd.data_ptr() + 4 * off, yd.data_ptr() + 4 * off, od.data_ptr() + 4 * off, bq,
                       gpuh2h.QUERY_LCA, sp)
        b.record(stream)
    torch.cuda.synchronize()
    lat_dev = [a.elapsed_time(b) * 1000.0 for a, b in ev]
    lat_e2e = []
    for i in range(batches):
        off = (i * bq) % (nq - bq)
        s = time.perf_counter()
        g.query_host_ptr(xh.data_ptr() + 4 * off, yh.data_ptr() + 4 * off, oh.data_ptr() + 4 * off, bq,
                         gpuh2h.QUERY_LCA)
        lat_e2e.append((time.perf_counter() - s) * 1e6)
    return {"device_p50": pct(lat_dev, 50), "device_p99": pct(lat_dev, 99), "e2e_p50": pct(lat_e2e, 50),
            "e2e_p99": pct(lat_e2e, 99), "batches": batches}


def server_latency(g, n: int, slots: int = 4) -> dict:
    """10^5-pair requests of uniform pairs through the continuous-batching
    server (h2h_server_*), one and four in flight (closed loop); latency runs
    from each request's submission to its answers in host memory.  Parity:
    the server's answers equal the host batch API's."""
    import gpuh2h
    srv = gpuh2h.Server(slots=slots, slot_pairs=1 << 17)
    gid = srv.add(g)
    x, y = gpuh2h.uniform_pairs(n, 50_000, 900)
    out = np.zeros(len(x), np.int32)
    r = srv.submit(gid, x, y, out)
    srv.wait(r)
    srv.release(r)
    assert np.array_equal(out, g.query(x, y)), "server answers differ from the batch API"
    res = {}
    for inflight in (1, 4):
        srv.reset_stats()
        r = srv.load([gid], [n], rate=0, size_lo=100_000, size_hi=100_000, requests=300, inflight=inflight,
                     seed=31 + inflight)
        st = srv.stats()
        res["inflight%d" % inflight] = {"requests": r["requests"], "p50_us": pct(r["latency_us"], 50),
                                        "p99_us": pct(r["latency_us"], 99),
                                        "queries_per_s": r["pairs"] / r["wall_s"],
                                        "kernel_us_per_batch": st["kernel_us"] / max(1, st["batches"])}
    srv.close()
    res["what"] = ("300 requests of 1e5 uniform pairs, closed loop, %d server slots; parity: server answers equal "
                   "h2h_query_batch_host" % slots)
    return res


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


def small_graph_run(name: str, threads: int, steps: int, build_reps: int, plain_node_fill: bool) -> dict:
    """A second graph of the same generator family, as an extra key: build
    (median of build_reps), queries/s on 2e6-pair steps, the reference's GPU
    fill mappings on the same tree, and a Dijkstra check."""
    import torch

    import gpuh2h
    root = tempfile.mkdtemp(prefix="h2h_%s_" % name)
    files, arcs = gen_graph(root, name)
    H = WORKLOADS[name]["partition_height"]
    times, g = [], None
    for _ in range(max(1, build_reps)):
        if g is not None:
            g.close()
        torch.cuda.synchronize()
        g, bt = build_index(files, threads, H, name=name)
        times.append(bt)
    info = g.info()
    x, y = query_pairs(g, info["n"], 7)
    nq = len(x)
    xd, yd = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    od = torch.empty_like(xd)
    timed_queries(g, xd, yd, od, nq, 3, gpuh2h.QUERY_LCA)
    t = timed_queries(g, xd, yd, od, nq, steps, gpuh2h.QUERY_LCA)
    peak, _ = hbm_peak()
    b_step = algorithmic_bytes(g, x, y)
    fill_s = info["t_fill_gpu_us"] / 1e6
    fill_bytes = 8 * info["label_size"] + 8 * info["pos_size"] + 4 * info["label_updates"]
    plain_fill_ms, plain_fill_bad = g.fill_labels_plain("pair")
    assert plain_fill_bad == 0, "the plain fill mapping disagrees with the labels"
    fill = {"kernel": "fill_flow_kernel", "updates": info["label_updates"], "seconds": fill_s,
            "plain_gpu_seconds": plain_fill_ms / 1e3,
            "plain_gpu": "the reference's mapping: one thread per (v,u) pair, one launch + sync per tree level",
            "updates_per_s": info["label_updates"] / fill_s if fill_s > 0 else None,
            "algorithmic_bytes": fill_bytes, "achieved_gbs": fill_bytes / fill_s / 1e9 if fill_s > 0 else None,
            "frac_of_hbm": fill_bytes / fill_s / 1e9 / peak if fill_s > 0 else None}
    if plain_node_fill:
        node_fill_ms, node_fill_bad = g.fill_labels_plain("node")
        assert node_fill_bad == 0, "the node-per-thread fill mapping disagrees with the labels"
        fill.update({"plain_node_gpu_seconds": node_fill_ms / 1e3,
                     "plain_node_gpu": "the reference's parallelFine=1 mapping: one thread per node"})
    rng = np.random.default_rng(11)
    dij = dijkstra_check(files, g, info["n"], rng.choice(info["n"], 4, replace=False))
    assert dij["mismatches_lca"] == 0 and dij["mismatches_nolca"] == 0, "answers differ from Dijkstra"
    out = {"workload": DESCRIBE[name] % arcs, "build_s": statistics.median(times), "build_s_min": min(times),
           "build_phases_ms": phases_ms(info), "queries_per_s": steps * nq / t, "queries_per_step": nq,
           "roofline_frac": b_step / (t / steps) / 1e9 / peak, "label_fill": fill,
           "index": {"tree_height": info["tree_height"], "label_entries": info["label_size"],
                     "device_bytes": info["device_bytes"]},
           "parity": dij}
    g.close()
    shutil.rmtree(root, ignore_errors=True)
    return out


def cpu_baseline_run(threads: int, budget_s: float) -> dict:
    """The reference's CPU algorithm (oracle restatement) on the host cores,
    on the CPU workload: build, then the threaded UsingLCA query loop over the
    same kind of 2e6-pair batch for about budget_s seconds."""
    from oracle import oracle
    root = tempfile.mkdtemp(prefix="h2h_cpu_")
    try:
        oracle.generate_road(root, CPU_WORKLOAD, **WORKLOADS[CPU_WORKLOAD])
        files = files_for(root, CPU_WORKLOAD)
        H = WORKLOADS[CPU_WORKLOAD]["partition_height"]
        t0 = time.perf_counter()
        o = oracle.OracleGraph(*files, H, C_HEIGHT, threads).contract()
        t1 = time.perf_counter()
        o.build_labels(l4=True, threads=threads)
        t2 = time.perf_counter()
        x, y = oracle.uniform_pairs(o.n, Q_UNIFORM, 7)
        lx, ly = o.local_pairs(Q_LOCAL, LOCAL_HOPS, 7 + 1000)
        x, y = np.concatenate([x, lx]), np.concatenate([y, ly])
        done, q_time, reps = 0, 0.0, 0
        while q_time < budget_s and reps < 50:
            s = time.perf_counter()
            o.query_batch(x, y, lca=True, threads=threads)
            q_time += time.perf_counter() - s
            done += len(x)
            reps += 1
        o.close()
    finally:
        shutil.rmtree(root, ignore_errors=True)
    return dict(contract_s=t1 - t0, labels_s=t2 - t1, query_s=q_time, queries=done, reps=reps, nq=len(x))


def plain_gpu_reference_run(threads: int) -> dict:
    """The reference's own GPU path beside this library's: its unmodified G2H
    command line, built for sm_103a from the staged sources
    (oracle/build_ref_gpu.sh), and this library's G2H, both as
    `G2H cfg0 6 1 T 1 1 2 1` on the same seeded 4,096-vertex graph, each run
    timed by its own CSV timers (microseconds): TDInGPUTime = partition
    contraction, TDInCPUTime = global order, H2HUsingTime_GPU = GPU label fill
    (the shipped L3 labels), GPU*-256 = one batch of 1e6 uniform pairs.  The
    larger graphs are beyond it: it contracts each cell with one GPU thread
    that bubble-sorts the cell before every pick, cubic in a cell's size."""
    from gpuh2h import _build

    from oracle import oracle
    from oracle import plain_gpu_reference as pgr
    if not oracle.build_ref_gpu():
        return {"unavailable": "the reference's sources are not staged on this machine"}
    import gpuh2h
    params, H, C = pgr.GRAPHS["cfg0"]
    with tempfile.TemporaryDirectory() as rr, tempfile.TemporaryDirectory() as ro:
        oracle.generate_road(rr, "cfg0", **params)
        gpuh2h.generate_road(ro, "cfg0", **params)
        env = dict(os.environ)
        ref = pgr.run_cli(os.path.join(pgr.HERE, "_ref", "G2H_ref"), rr, "cfg0", H, C, threads, env)
        ours = pgr.run_cli(_build.CLI, ro, "cfg0", H, C, threads, dict(env, H2H_LABEL="L3"))
    return {"graph": "cfg0 (4,096 vertices, H=6, C=1)", "reference": ref, "ours": ours,
            "what": "the reference's unmodified G2H (nvcc sm_103a) and this library's G2H, same graph and "
                    "arguments `G2H cfg0 6 1 T 1 1 2 1`; microseconds from each run's own CSV timers"}


def files_for(root: str, name: str):
    pre = os.path.join(root, "Partition", name, "Latitude")
    return (os.path.join(root, "Graph", "USA", name + "Edge.txt"), pre + "ID.txt", pre + "Cut.txt")


def run_reference_arm(args) -> int:
    """The reference's CPU path (oracle restatement, all host threads) on the
    CPU workload; this process loads the oracle library only."""
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    from oracle import oracle
    threads = os.cpu_count() or 1
    root = tempfile.mkdtemp(prefix="h2h_ref_")
    try:
        arcs = oracle.generate_road(root, CPU_WORKLOAD, **WORKLOADS[CPU_WORKLOAD])
        files = files_for(root, CPU_WORKLOAD)
        H = WORKLOADS[CPU_WORKLOAD]["partition_height"]
        t0 = time.perf_counter()
        o = oracle.OracleGraph(*files, H, C_HEIGHT, threads).contract()
        t1 = time.perf_counter()
        o.build_labels(l4=True, threads=threads)
        t2 = time.perf_counter()
        # the same pairs as the GPU arm draws on this graph (seed 7)
        ux, uy = oracle.uniform_pairs(o.n, Q_UNIFORM, 7)
        lx, ly = o.local_pairs(Q_LOCAL, LOCAL_HOPS, 7 + 1000)
        x, y = np.concatenate([ux, lx]), np.concatenate([uy, ly])
        for _ in range(args.warmup):
            o.query_batch(x, y, lca=True, threads=threads)
        times = []
        for _ in range(args.steps):
            s = time.perf_counter()
            o.query_batch(x, y, lca=True, threads=threads)
            times.append(time.perf_counter() - s)
        o.close()
    finally:
        shutil.rmtree(root, ignore_errors=True)
    total = sum(times)
    value = args.steps * len(x) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": (DESCRIBE[CPU_WORKLOAD] % arcs).replace("GPU contraction + GPU L4 labels",
                                                                        "CPU contraction + CPU L4 labels")
                   + "; step = 2e6 queries (1e6 uniform + 1e6 local <=20 hops), UsingLCA",
                   "why_not_road6m": "the 6,262,104-vertex graph is beyond a bounded CPU run: the reference's "
                                     "partition contraction (restated per cell with its bubble sorts, cubic in "
                                     "the cell's size) and a 117 GB label fill on the host",
                   "parallelism": "host threads"},
        "build_s": t2 - t0, "build_phases_s": {"contract": t1 - t0, "labels": t2 - t1},
        "cpu_baseline": {"value": value, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": "%d steps x %d queries on %s, UsingLCA, %d threads" % (
                             args.steps, len(x), CPU_WORKLOAD, threads)},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_serving(args) -> int:
    """Serving: the 6,262,104-vertex road graph resident with 8 road graphs of
    50k-1M vertices in one continuous-batching server; Poisson request
    streams (1-10^5 pairs per request, log-uniform, random graph) at
    10^3-10^5 requests/s, latency of 10^5-pair requests on the large graph,
    and closed-loop throughput against the HBM roofline of the query kernel."""
    import torch

    import gpuh2h
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    threads = max(1, os.cpu_count() or 1)
    root = tempfile.mkdtemp(prefix="h2h_serve_")
    specs = [("road6m", WORKLOADS["road6m"])]
    for i, p in enumerate(gpuh2h.road_batch_params(8, 50_000, 1_000_000, seed=23)):
        specs.append(("res%d" % i, p))
    graphs, build = [], []
    for name, p in specs:
        t0 = time.perf_counter()
        arcs = gpuh2h.generate_road(root, name, **p)
        t_gen = time.perf_counter() - t0
        g, bt = build_index(gpuh2h.files_for(root, name), threads, H=p["partition_height"], name=name)
        i = g.info()
        build.append({"graph": name, "vertices": i["n"], "arcs": arcs, "partition_height": p["partition_height"],
                      "build_s": bt, "gen_s": t_gen, "tree_height": i["tree_height"],
                      "label_entries": i["label_size"], "device_gb": i["device_bytes"] / 1e9,
                      "phases_ms": phases_ms(i)})
        log("built %s: %d vertices, %.1f s, %.1f GB" % (name, i["n"], bt, i["device_bytes"] / 1e9))
        graphs.append(g)
    nv = [g.info()["n"] for g in graphs]
    srv = gpuh2h.Server(slots=args.serve_slots, slot_pairs=1 << 17)
    gids = [srv.add(g) for g in graphs]
    for k, g in enumerate(graphs):
        x, y = gpuh2h.uniform_pairs(nv[k], 50_000, 900 + k)
        out = np.zeros(len(x), np.int32)
        r = srv.submit(gids[k], x, y, out)
        srv.wait(r)
        srv.release(r)
        assert np.array_equal(out, g.query(x, y)), "server answers differ on graph %d" % k
    runs = {}
    for inflight in (1, 4):
        srv.reset_stats()
        r = srv.load([gids[0]], [nv[0]], rate=0, size_lo=100_000, size_hi=100_000, requests=300,
                     inflight=inflight, seed=31 + inflight)
        st = srv.stats()
        runs["big_1e5_inflight%d" % inflight] = {
            "requests": r["requests"], "p50_us": pct(r["latency_us"], 50), "p99_us": pct(r["latency_us"], 99),
            "queries_per_s": r["pairs"] / r["wall_s"], "kernel_us_per_batch": st["kernel_us"] / max(1, st["batches"])}
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
    srv.reset_stats()
    r = srv.load([gids[0]], [nv[0]], rate=0, size_lo=100_000, size_hi=100_000, requests=600, inflight=16, seed=77)
    st = srv.stats()
    xs, ys = gpuh2h.uniform_pairs(nv[0], 200_000, 4242)
    b_q = algorithmic_bytes(graphs[0], xs, ys) / len(xs)
    peak, peak_src = hbm_peak()
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="road6m", choices=sorted(WORKLOADS))
    ap.add_argument("--build-reps", type=int, default=2)
    ap.add_argument("--latency-batches", type=int, default=200)
    ap.add_argument("--cpu-budget", type=float, default=10.0, help="seconds of CPU query work for cpu_baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the 264k-vertex graph and the 64-graph batch")
    ap.add_argument("--dijkstra-sources", type=int, default=3)
    ap.add_argument("--plain-node-fill", action="store_true",
                    help="also time the reference's node-per-thread fill mapping on the small graph (a minute)")
    ap.add_argument("--batch-graphs", type=int, default=64, help="graphs of the batched-build measurement (0: skip)")
    ap.add_argument("--serve", action="store_true", help="run the full serving measurement instead")
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-seconds", type=float, default=2.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.serve:
        return run_serving(args)

    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import gpuh2h
    threads = max(1, (os.cpu_count() or 1) // max(1, world))
    name = args.workload
    H = WORKLOADS[name]["partition_height"]
    root = tempfile.mkdtemp(prefix="h2h_bench_%d_" % rank)
    t0 = time.perf_counter()
    files, arcs = gen_graph(root, name)
    gen_s = time.perf_counter() - t0
    # ---- build (whole H2H construction from the loaded files)
    build_times, g = [], None
    for r in range(max(1, args.build_reps)):
        if g is not None:
            g.close()
        torch.cuda.synchronize()
        g, bt = build_index(files, threads, H, name=name)
        build_times.append(bt)
        log("build %d: %.2f s" % (r, bt))
    info = g.info()
    n = info["n"]
    x, y = query_pairs(g, n, rank_query_seed(rank))
    nq = len(x)
    xd = torch.from_numpy(x).cuda()
    yd = torch.from_numpy(y).cuda()
    od = torch.empty_like(xd)
    sp = torch.cuda.current_stream().cuda_stream
    for _ in range(args.warmup):
        g.query_device(xd.data_ptr(), yd.data_ptr(), od.data_ptr(), nq, gpuh2h.QUERY_LCA, sp)
    torch.cuda.synchronize()
    od2 = torch.empty_like(xd)
    g.query_device(xd.data_ptr(), yd.data_ptr(), od2.data_ptr(), nq, gpuh2h.QUERY_NOLCA, sp)
    torch.cuda.synchronize()
    assert torch.equal(od, od2), "UsingLCA and noLCA answers differ"
    # ---- timed region: K steps, device-resident inputs
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    t_local = timed_queries(g, xd, yd, od, nq, args.steps, gpuh2h.QUERY_LCA)
    barrier(world)
    clocks = sampler.stop()
    t_max = reduce_max(t_local, world)
    value = world * args.steps * nq / t_max
    kernel_s = t_local / args.steps
    # ---- roofline of the query kernel (one launch per step)
    abytes = algorithmic_bytes(g, x, y)
    peak, peak_src = hbm_peak()
    achieved = abytes / kernel_s / 1e9
    traffic, traffic_src = None, None
    tf = os.path.join(REPO, "profiles", "query_traffic.json")
    if os.path.exists(tf):
        try:
            rec = json.load(open(tf)).get(name)
            if rec:
                traffic = rec["dram_bytes_per_query"] * nq
                traffic_src = ("not measured in this run: ncu dram__bytes_read.sum + dram__bytes_write.sum per query "
                               "of one query_tile_kernel launch on this workload (profiles/query_traffic.json) x "
                               "queries per step")
        except Exception:
            traffic = None
    # ---- the reference's one-thread-per-query mapping on the same index
    g.query_device_plain(xd.data_ptr(), yd.data_ptr(), od2.data_ptr(), nq, gpuh2h.QUERY_LCA, sp)
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps_plain = max(3, min(args.steps, 20))
    stream = torch.cuda.current_stream()
    p0.record(stream)
    for _ in range(reps_plain):
        g.query_device_plain(xd.data_ptr(), yd.data_ptr(), od2.data_ptr(), nq, gpuh2h.QUERY_LCA, sp)
    p1.record(stream)
    torch.cuda.synchronize()
    plain_value = reps_plain * nq / (p0.elapsed_time(p1) / 1000.0)
    assert torch.equal(od, od2), "the plain mapping's answers differ"
    # ---- e2e through the public host-buffer C ABI call (pinned host buffers)
    xh = torch.from_numpy(x).pin_memory()
    yh = torch.from_numpy(y).pin_memory()
    oh = torch.empty(nq, dtype=torch.int32).pin_memory()
    for _ in range(args.warmup):
        g.query_host_ptr(xh.data_ptr(), yh.data_ptr(), oh.data_ptr(), nq, gpuh2h.QUERY_LCA)
    barrier(world)
    s = time.perf_counter()
    for _ in range(args.steps):
        g.query_host_ptr(xh.data_ptr(), yh.data_ptr(), oh.data_ptr(), nq, gpuh2h.QUERY_LCA)
    e2e_local = time.perf_counter() - s
    e2e_t = reduce_max(e2e_local, world)
    e2e_value = world * args.steps * nq / e2e_t
    assert np.array_equal(oh.numpy(), od.cpu().numpy())
    # ---- latency of 10^5-pair batches, and through the server
    latency = latency_runs(g, xd, yd, od, xh, yh, oh, nq, args.latency_batches)
    serving = server_latency(g, n) if rank == 0 else None
    # ---- parity: Dijkstra from sampled sources to every vertex
    parity = None
    if rank == 0 and args.dijkstra_sources > 0:
        rng = np.random.default_rng(5)
        parity = dijkstra_check(files, g, n, rng.choice(n, args.dijkstra_sources, replace=False))
        assert parity["mismatches_lca"] == 0 and parity["mismatches_nolca"] == 0, "answers differ from Dijkstra"
    fill_s = info["t_fill_gpu_us"] / 1e6
    fill_bytes = 8 * info["label_size"] + 8 * info["pos_size"] + 4 * info["label_updates"]
    fill = {"kernel": "fill_flow_kernel", "updates": info["label_updates"], "seconds": fill_s,
            "updates_per_s": info["label_updates"] / fill_s if fill_s > 0 else None,
            "algorithmic_bytes": fill_bytes, "achieved_gbs": fill_bytes / fill_s / 1e9 if fill_s > 0 else None,
            "frac_of_hbm": fill_bytes / fill_s / 1e9 / peak if fill_s > 0 else None}
    index = {"tree_height": info["tree_height"], "label_entries": info["label_size"],
             "label_gb": info["label_size"] * 4 / 1e9, "device_bytes": info["device_bytes"],
             "max_label": info["max_label"]}
    g.close()
    del xd, yd, od, od2
    torch.cuda.empty_cache()
    shutil.rmtree(root, ignore_errors=True)
    # ---- extra keys (rank 0, N=1): the 264k-vertex graph and the 64-graph batch
    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        if name != "cfg1":
            extras["cfg1"] = small_graph_run("cfg1", threads, min(args.steps, 20), 3, args.plain_node_fill)
        if args.batch_graphs > 0:
            extras["batched_build"] = batched_build(threads, args.batch_graphs)
    # ---- CPU baseline (rank 0, N=1): the reference's CPU algorithm on host cores
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        cb = cpu_baseline_run(cores, args.cpu_budget)
        cpu = {"value": cb["queries"] / cb["query_s"], "unit": "queries/s", "cores": cores, "kind": "port",
               "sample": "%s (264,346 vertices; the 6,262,104-vertex graph is beyond a bounded CPU run): %d x %d "
                         "queries (UsingLCA, L4 labels) over %d host threads; oracle build %.1f s (contract %.1f s "
                         "+ labels %.1f s)" % (CPU_WORKLOAD, cb["reps"], cb["nq"], cores,
                                               cb["contract_s"] + cb["labels_s"], cb["contract_s"], cb["labels_s"]),
               "build_s": cb["contract_s"] + cb["labels_s"]}
    # ---- the reference's own GPU path on the graph it can contract in seconds
    plain_ref = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and not args.no_extras:
        plain_ref = plain_gpu_reference_run(os.cpu_count() or 1)
    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": DESCRIBE[name] % arcs + "; step = 2e6 queries (1e6 uniform + 1e6 local <=20 hops), "
                               "UsingLCA",
                   "queries_per_step": nq, "l2": "index %.1f GB resident > L2 (no flush)" % (info["device_bytes"] / 1e9),
                   "parallelism": "replicas x%d (queries sharded by rank)" % world},
        "gen_s": gen_s, "build_s": statistics.median(build_times), "build_s_min": min(build_times),
        "build_phases_ms": phases_ms(info), "label_fill": fill, "index": index,
        "latency_us_1e5": latency, "serving_1e5": serving,
        "plain_gpu": {"value": plain_value, "unit": "queries/s",
                      "what": "one thread per query (the reference's mapping) on the same index"},
        "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": 8 * nq, "d2h_bytes_per_step": 4 * nq,
                "what": "h2h_query_batch_host from pinned host buffers, %d steps" % args.steps},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": traffic_src, "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": abytes, "kernel": "query_tile_kernel<LCA>"},
        "clocks": clocks,
        "parity": parity,
        "cpu_baseline": cpu,
        "plain_gpu_reference": plain_ref,
    }
    line.update(extras)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
