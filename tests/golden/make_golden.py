"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs the CPU-only build of the reference's own translation units
(oracle/build_ref.sh -> oracle/_ref/ref_harness_{L3,L4}) on
  * the reference's 13-vertex sample graph under its four partitions
    (Graph/USA/13Edge.txt, Partition/13/*), every ChangeToGlobalHeight;
  * the seeded 64x64 road-like grid written by the library's generator,
    ChangeToGlobalHeight 1, 2 and 6;
and stores inputs (13-vertex case) and outputs as compressed .npz files.
Large arrays of the 64x64 case are stored as SHA-256 digests plus samples.
It also checks that the C oracle (oracle/h2h_oracle.c) reproduces every
array, so the fixtures pin both.

Usage (needs the reference tree; REF or --ref names it):
    REF=<reference tree> python tests/golden/make_golden.py
"""
from __future__ import annotations

import argparse
import hashlib
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "gpu-h2h_gb300"))

from oracle import oracle as O  # noqa: E402

PARTS = [("Latitude", 4), ("Minimum", 4), ("metis", 3), ("scotch", 3)]
CFG0 = dict(name="cfg0", H=6, Cs=(1, 2, 6), nq=20000, seed=5)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def oracle_arrays(e, i, c, H, C, l4, pairs):
    g = O.OracleGraph(e, i, c, H, C, 4).contract().build_labels(l4=l4)
    lab = g.labels()
    rh, ri = g.rmq()
    tb, th = g.bfs()
    out = dict(order=g.order(), father=g.father(), depth=g.depth(), first=g.first(), rmq_hash=rh, rmq_id=ri,
               tree_bfs=tb, tree_hash=th, **lab)
    out["q_lca"] = g.query_batch(pairs[:, 0], pairs[:, 1])
    out["q_nolca"] = g.query_batch(pairs[:, 0], pairs[:, 1], lca=False)
    return out


def compare(ref: dict, orc: dict, what: str):
    for k in ("order", "father", "depth", "first", "rmq_hash", "rmq_id", "dis_hash", "dis", "pos_hash", "pos_id",
              "pos_pos", "tree_bfs", "tree_hash", "q_lca", "q_nolca"):
        if not np.array_equal(ref[k], orc[k]):
            raise SystemExit("oracle differs from the reference on %s: %s" % (what, k))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("REF"), help="the reference tree (default: $REF)")
    args = ap.parse_args()
    if not args.ref:
        raise SystemExit("make_golden.py: name the reference tree with --ref or REF")
    env = dict(os.environ, REF=args.ref)
    subprocess.check_call([os.path.join(REPO, "oracle", "build_ref.sh")], env=env)
    # 13-vertex sample: copy the input files next to the fixtures
    sample = os.path.join(HERE, "sample13")
    os.makedirs(os.path.join(sample, "Graph", "USA"), exist_ok=True)
    os.makedirs(os.path.join(sample, "Partition", "13"), exist_ok=True)
    shutil.copyfile(os.path.join(args.ref, "Graph/USA/13Edge.txt"), os.path.join(sample, "Graph/USA/13Edge.txt"))
    for meth, _ in PARTS:
        for kind in ("ID", "Cut"):
            shutil.copyfile(os.path.join(args.ref, "Partition/13/%s%s.txt" % (meth, kind)),
                            os.path.join(sample, "Partition/13/%s%s.txt" % (meth, kind)))
    pairs13 = np.array([[a, b] for a in range(13) for b in range(13)], np.int32)
    store = {}
    for meth, H in PARTS:
        e = os.path.join(sample, "Graph/USA/13Edge.txt")
        i = os.path.join(sample, "Partition/13/%sID.txt" % meth)
        c = os.path.join(sample, "Partition/13/%sCut.txt" % meth)
        for C in range(1, H + 1):
            for l4 in (True, False):
                ref = O.run_reference(e, i, c, H, C, 2, l4=l4, pairs=pairs13)
                compare(ref, oracle_arrays(e, i, c, H, C, l4, pairs13), "13/%s/C%d/%s" % (meth, C, l4))
                tag = "13_%s_C%d_%s" % (meth, C, "L4" if l4 else "L3")
                for k, v in ref.items():
                    store[tag + "/" + k] = v
    store["pairs13"] = pairs13
    np.savez_compressed(os.path.join(HERE, "sample13.npz"), **store)
    # 64x64 grid from the library's generator
    import gpuh2h
    with tempfile.TemporaryDirectory() as root:
        gpuh2h.generate_road(root, CFG0["name"])
        e, i, c = gpuh2h.files_for(root, CFG0["name"])
        files = {os.path.basename(p): open(p, "rb").read() for p in (e, i, c)}
        rng = np.random.default_rng(CFG0["seed"])
        pairs = np.stack([rng.integers(0, 4096, CFG0["nq"]), rng.integers(0, 4096, CFG0["nq"])], 1).astype(np.int32)
        g0 = {"pairs": pairs}
        for name, data in files.items():
            g0["file_sha256/" + name] = np.frombuffer(hashlib.sha256(data).digest(), np.uint8)
        for C in CFG0["Cs"]:
            for l4 in (True, False):
                ref = O.run_reference(e, i, c, CFG0["H"], C, 4, l4=l4, pairs=pairs)
                compare(ref, oracle_arrays(e, i, c, CFG0["H"], C, l4, pairs), "cfg0/C%d/%s" % (C, l4))
                tag = "cfg0_C%d_%s" % (C, "L4" if l4 else "L3")
                for k in ("order", "father", "depth", "first", "gpu_vertices", "q_lca", "q_nolca", "tree_hash"):
                    g0[tag + "/" + k] = ref[k]
                for k in ("rmq_hash", "rmq_id", "dis_hash", "dis", "pos_hash", "pos_id", "pos_pos", "tree_bfs",
                          "adj_hash", "adj_id", "adj_w"):
                    g0[tag + "/sha256/" + k] = np.frombuffer(bytes.fromhex(digest(ref[k])), np.uint8)
                    g0[tag + "/len/" + k] = np.array([len(ref[k])], np.int64)
                g0[tag + "/dis_sample"] = ref["dis"][::97]
        # the same grid with parallel arcs (tests/conftest.py:write_multigraph)
        sys.path.insert(0, os.path.join(REPO, "tests"))
        from conftest import write_multigraph
        mfiles = write_multigraph(root)
        for C in (1, 2):
            ref = O.run_reference(*mfiles, CFG0["H"], C, 4, l4=True, pairs=pairs)
            compare(ref, oracle_arrays(*mfiles, CFG0["H"], C, True, pairs), "multi/C%d" % C)
            tag = "multi_C%d_L4" % C
            for k in ("order", "father", "q_lca", "q_nolca"):
                g0[tag + "/" + k] = ref[k]
            for k in ("dis", "adj_id", "adj_w", "rmq_id", "pos_pos"):
                g0[tag + "/sha256/" + k] = np.frombuffer(bytes.fromhex(digest(ref[k])), np.uint8)
    np.savez_compressed(os.path.join(HERE, "cfg0.npz"), **g0)
    print("wrote", os.path.join(HERE, "sample13.npz"), os.path.join(HERE, "cfg0.npz"))


if __name__ == "__main__":
    main()
