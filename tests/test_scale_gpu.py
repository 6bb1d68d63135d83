"""Parity at the benchmarked scales, on the inputs where the large-graph code
paths switch on by themselves (no forcing through environment variables).

* The 264,346-vertex road graph (H = 10, C = 2): the elimination picks its
  cluster sizes and cooperative steps from its cost model and stages long
  lists in global memory; the fill cuts the wide top separators into tiles
  combined with atomicMin.  Everything is compared with the oracle, which is
  pinned to the reference's own CPU build by the golden fixtures: the
  elimination order, the tree, the Euler tour and sparse table, every label
  and position entry, and 2e5 query answers in both modes.
* A 1,000,000-vertex road graph (H = 12) whose tree is deeper than 2,048
  levels, so the fill takes its deep-tree tile preset: every answer from
  sampled sources to all vertices equals the oracle's Dijkstra.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CFG1 = dict(n=264346, target_arcs=733846, aspect_milli=1300, jitter_milli=300, diag_permille=50, hw_tiers=1,
            hw_permille10=50, hw_k=3, hw_scale_milli=400, partition_height=10, seed=1, cols=0, drop_permille=0)
DEEP = dict(n=1000000, target_arcs=2776000, aspect_milli=1300, jitter_milli=300, diag_permille=50, hw_tiers=1,
            hw_permille10=50, hw_k=3, hw_scale_milli=400, partition_height=12, seed=5, cols=0, drop_permille=0)


def _gpu_build(files, H, C):
    import gpuh2h
    g = gpuh2h.Graph("t", H, C, os.cpu_count() or 4, 1, files=files)
    g.contraction_noHub(1)
    g.constructLabel_noHub(2, 1, gpuh2h.LABEL_L4)
    return g


def test_cfg1_road_graph_matches_oracle(tmp_path):
    import gpuh2h
    from oracle import oracle
    root = str(tmp_path)
    gpuh2h.generate_road(root, "cfg1", **CFG1)
    files = gpuh2h.files_for(root, "cfg1")
    g = _gpu_build(files, 10, 2)
    o = oracle.OracleGraph(*files, 10, 2, os.cpu_count() or 4).contract().build_labels(l4=True)
    assert g.info()["gpu_vertices"] == o.summary()["gpu_vertices"]
    assert np.array_equal(g.order(), o.order()), "elimination order"
    f, d, fi = g.tree()
    assert np.array_equal(f, o.father()), "father"
    assert np.array_equal(d, o.depth()), "depth"
    assert np.array_equal(fi, o.first()), "first appearance"
    for a, b, k in zip(g.rmq(), o.rmq(), ("rmq_hash", "rmq_id")):
        assert np.array_equal(a, b), k
    for a, b, k in zip(g.bfs(), o.bfs(), ("tree_bfs", "tree_hash")):
        assert np.array_equal(a, b), k
    ga, oa = g.labels(), o.labels()
    for k in ("dis_hash", "pos_hash", "pos_id", "pos_pos", "dis"):
        if not np.array_equal(ga[k], oa[k]):
            bad = np.nonzero(ga[k] != oa[k])[0] if len(ga[k]) == len(oa[k]) else []
            pytest.fail("%s differs (%d entries, first %s)" % (k, len(bad), bad[:5]))
    del ga, oa
    x, y = gpuh2h.uniform_pairs(g.info()["n"], 100_000, 21)
    lx, ly = g.local_pairs(100_000, 20, 22)
    x, y = np.concatenate([x, lx]), np.concatenate([y, ly])
    for mode, lca in ((gpuh2h.QUERY_LCA, True), (gpuh2h.QUERY_NOLCA, False)):
        assert np.array_equal(g.query(x, y, mode), o.query_batch(x, y, lca=lca)), "answers (lca=%s)" % lca
    g.close()
    o.close()


def test_deep_tree_road_graph_matches_dijkstra(tmp_path):
    import gpuh2h
    from oracle import oracle
    root = str(tmp_path)
    gpuh2h.generate_road(root, "deep", **DEEP)
    files = gpuh2h.files_for(root, "deep")
    g = _gpu_build(files, 12, 2)
    info = g.info()
    assert info["tree_height"] > 2048, "the graph no longer selects the deep-tree fill preset"
    n = info["n"]
    o = oracle.OracleGraph(*files, 12, 2, 4)
    rng = np.random.default_rng(3)
    y = np.arange(n, dtype=np.int32)
    for s in rng.choice(n, 3, replace=False):
        ref = o.dijkstra(int(s))
        x = np.full(n, s, np.int32)
        for mode in (gpuh2h.QUERY_LCA, gpuh2h.QUERY_NOLCA):
            got = g.query(x, y, mode)
            bad = np.nonzero(got != ref)[0]
            assert len(bad) == 0, "source %d mode %d: %d targets differ, first %s" % (s, mode, len(bad), bad[:5])
    g.close()
    o.close()
