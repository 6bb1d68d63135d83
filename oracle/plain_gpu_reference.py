"""The reference's own GPU path timed beside this library on the same inputs.

MEASUREMENT INFRASTRUCTURE, not product code: it runs the reference's
unmodified G2H command line built for sm_103a (oracle/build_ref_gpu.sh:
`G2H <G> H C T 1 1 2 1`, GPU partition contraction, GPU LL label fill with the
shipped L3 labels, GPU batched queries) and this library's G2H with the same
arguments (L3 and L4 labels) in separate working directories holding the same
seeded graph, and reads each run's own timers from the CSV files both write
(ConstructInfo/<G>/constructInfo.csv: Graph_Fundamental.cu:148;
QueryResult/<G>/random.csv: Query.cu:608).  It also runs the reference's GPU
harness with the L4 label kernel (kernel_functions.cu:739-743 enabled) for an
L4-to-L4 label-fill time.

The graphs stay small: the reference eliminates each partition cell with one
GPU thread that bubble-sorts the cell's candidates before every pick
(kernel_functions.cu:309-479), so its contraction time grows with the cube of
a cell's size (the 264,346-vertex graph's largest cell costs 5.4 s of one CPU
core in the oracle's restatement of that body).

    python oracle/plain_gpu_reference.py [--graphs cfg0,grid128] > out.json
"""
from __future__ import annotations

import argparse
import csv
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
# run as a script, this directory heads sys.path and would shadow the
# oracle package with oracle.py
sys.path[:] = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
for _p in (REPO, os.path.join(REPO, "gpu-h2h_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

GRAPHS = {
    # name: (generator parameters, partition height, ChangeToGlobalHeight)
    "cfg0": ({}, 6, 1),
    "grid128": (dict(n=16384, cols=128, partition_height=8, seed=77), 8, 1),
}
COLUMNS = ("TDInGPUTime", "TDInCPUTime", "H2HmallocTime", "H2HConstructBFSTreeTime", "H2HUsingTime_CPU",
           "H2HTranslateTime", "H2HUsingTime_GPU")
QUERY_COLUMNS = ("GPUnoLCA-256", "GPUwithLCA-256")


def _last_row(path: str) -> dict:
    with open(path) as f:
        rows = list(csv.reader(f))
    head, row = rows[0], rows[-1]
    return {h: v for h, v in zip(head, row) if h}


def run_cli(exe: str, root: str, name: str, H: int, C: int, threads: int, env: dict) -> dict:
    for d in ("ConstructInfo/" + name, "QueryResult/" + name):
        os.makedirs(os.path.join(root, d), exist_ok=True)
    t0 = time.perf_counter()
    r = subprocess.run([exe, name, str(H), str(C), str(threads), "1", "1", "2", "1"], cwd=root, env=env,
                       capture_output=True, timeout=900)
    wall = time.perf_counter() - t0
    if r.returncode != 0:
        raise RuntimeError("%s failed (%d): %s" % (exe, r.returncode, r.stderr.decode()[-2000:]))
    ci = _last_row(os.path.join(root, "ConstructInfo", name, "constructInfo.csv"))
    qr = _last_row(os.path.join(root, "QueryResult", name, "random.csv"))
    out = {k: int(float(ci[k])) for k in COLUMNS if k in ci}
    out.update({k: int(float(qr[k])) for k in QUERY_COLUMNS if k in qr})
    out["queries"] = int(qr["queryNumber"])
    out["process_wall_s"] = wall
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--graphs", default="cfg0,grid128")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 4)
    args = ap.parse_args()
    from gpuh2h import _build

    from oracle import oracle
    if not oracle.build_ref_gpu():
        print(json.dumps({"unavailable": "the reference's sources are not staged on this machine"}))
        return 0
    _build.build()
    ref_exe = os.path.join(HERE, "_ref", "G2H_ref")
    res = {"what": "reference G2H (unmodified, nvcc sm_103a) vs this library's G2H, same seeded graph and "
                   "arguments `G2H <G> H C T 1 1 2 1`; times in microseconds from each run's own CSV timers "
                   "(TDInGPUTime = partition contraction, TDInCPUTime = global order, H2HUsingTime_GPU = GPU "
                   "label fill, GPU*-256 = one batch of 1e6 uniform pairs)", "graphs": {}}
    for name in args.graphs.split(","):
        params, H, C = GRAPHS[name]
        entry = {"H": H, "C": C}
        with tempfile.TemporaryDirectory() as rr, tempfile.TemporaryDirectory() as ro:
            n_arcs = oracle.generate_road(rr, name, **params)
            oracle.generate_road(ro, name, **params)
            entry["arcs"] = n_arcs
            env = dict(os.environ)
            entry["reference_L3"] = run_cli(ref_exe, rr, name, H, C, args.threads, env)
            print("reference %s: %s" % (name, entry["reference_L3"]), file=sys.stderr, flush=True)
            entry["ours_L3"] = run_cli(_build.CLI, ro, name, H, C, args.threads, dict(env, H2H_LABEL="L3"))
            entry["ours_L4"] = run_cli(_build.CLI, ro, name, H, C, args.threads, dict(env, H2H_LABEL="L4"))
            files = (os.path.join(rr, "Graph", "USA", name + "Edge.txt"),
                     os.path.join(rr, "Partition", name, "LatitudeID.txt"),
                     os.path.join(rr, "Partition", name, "LatitudeCut.txt"))
            got = oracle.run_reference(*files, H, C, threads=args.threads, l4=True, gpu=True)
            entry["reference_L4_harness"] = got["times"]
        res["graphs"][name] = entry
    print(json.dumps(res), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
