"""The C oracle against the golden fixtures generated by the reference itself.

tests/golden/make_golden.py ran the CPU build of the reference's own
translation units and stored its outputs; here the plain-C restatement
(oracle/h2h_oracle.c) must reproduce them exactly, which pins the oracle that
the GPU parity tests use as their checker.
"""
import hashlib

import numpy as np
import pytest

from conftest import PARTS, sample13_files
from oracle import oracle as O

KEYS = ("order", "father", "depth", "first", "rmq_hash", "rmq_id", "dis_hash", "dis", "pos_hash", "pos_id",
        "pos_pos", "tree_bfs", "tree_hash")


def _all(g, pairs):
    lab = g.labels()
    rh, ri = g.rmq()
    tb, th = g.bfs()
    return dict(order=g.order(), father=g.father(), depth=g.depth(), first=g.first(), rmq_hash=rh, rmq_id=ri,
                tree_bfs=tb, tree_hash=th, q_lca=g.query_batch(pairs[:, 0], pairs[:, 1]),
                q_nolca=g.query_batch(pairs[:, 0], pairs[:, 1], lca=False), **lab)


@pytest.mark.parametrize("meth,code,H", PARTS)
@pytest.mark.parametrize("l4", [True, False])
def test_sample13_every_change_height(golden13, meth, code, H, l4):
    pairs = golden13["pairs13"]
    for C in range(1, H + 1):
        tag = "13_%s_C%d_%s/" % (meth, C, "L4" if l4 else "L3")
        g = O.OracleGraph(*sample13_files(meth), H, C, 2).contract().build_labels(l4=l4)
        got = _all(g, pairs)
        for k in KEYS + ("q_lca", "q_nolca"):
            assert np.array_equal(got[k], golden13[tag + k]), (tag, k)


def _sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def test_generator_reproduces_fixture_files(cfg0_root, golden0):
    import gpuh2h
    for p in gpuh2h.files_for(cfg0_root, "cfg0"):
        name = p.rsplit("/", 1)[1]
        assert np.array_equal(_sha(np.frombuffer(open(p, "rb").read(), np.uint8)), golden0["file_sha256/" + name])


@pytest.mark.parametrize("C", [1, 2, 6])
@pytest.mark.parametrize("l4", [True, False])
def test_cfg0(cfg0_root, golden0, C, l4):
    import gpuh2h
    tag = "cfg0_C%d_%s/" % (C, "L4" if l4 else "L3")
    pairs = golden0["pairs"]
    g = O.OracleGraph(*gpuh2h.files_for(cfg0_root, "cfg0"), 6, C, 4).contract().build_labels(l4=l4)
    got = _all(g, pairs)
    for k in ("order", "father", "depth", "first", "q_lca", "q_nolca", "tree_hash"):
        assert np.array_equal(got[k], golden0[tag + k]), k
    for k in ("rmq_hash", "rmq_id", "dis_hash", "dis", "pos_hash", "pos_id", "pos_pos", "tree_bfs"):
        assert len(got[k]) == golden0[tag + "len/" + k][0], k
        assert np.array_equal(_sha(got[k]), golden0[tag + "sha256/" + k]), k
    ah, aid, aw = g.adj()
    for k, v in (("adj_hash", ah), ("adj_id", aid), ("adj_w", aw)):
        assert np.array_equal(_sha(v), golden0[tag + "sha256/" + k]), k
    assert g.summary()["gpu_vertices"] == golden0[tag + "gpu_vertices"][0]


def test_l4_labels_are_exact_distances(cfg0_root):
    """L4 rows hold exact shortest distances to every ancestor (Dijkstra)."""
    import gpuh2h
    g = O.OracleGraph(*gpuh2h.files_for(cfg0_root, "cfg0"), 6, 1, 4).contract().build_labels(l4=True)
    lab = g.labels()
    father, depth = g.father(), g.depth()
    for v in range(0, g.n, 257):
        d = g.dijkstra(v)
        row = lab["dis"][lab["dis_hash"][v]:lab["dis_hash"][v + 1]]
        a = v
        for j in range(depth[v] - 1, -1, -1):
            assert row[j] == d[a]
            a = father[a]


def test_l3_lca_query_is_inexact_but_nolca_exact(golden0):
    """The reference ships L3 labels; with them its UsingLCA query is inexact, noLCA exact."""
    l3 = golden0["cfg0_C1_L3/q_lca"]
    l4 = golden0["cfg0_C1_L4/q_lca"]
    assert (l3 != l4).any()
    assert np.array_equal(golden0["cfg0_C1_L3/q_nolca"], l4)


@pytest.mark.parametrize("C", [1, 2])
def test_multigraph(multi_files, golden0, C):
    tag = "multi_C%d_L4/" % C
    pairs = golden0["pairs"]
    g = O.OracleGraph(*multi_files, 6, C, 4).contract().build_labels(l4=True)
    assert np.array_equal(g.order(), golden0[tag + "order"])
    assert np.array_equal(g.father(), golden0[tag + "father"])
    assert np.array_equal(_sha(g.labels()["dis"]), golden0[tag + "sha256/dis"])
    ah, aid, aw = g.adj()
    assert np.array_equal(_sha(aw), golden0[tag + "sha256/adj_w"])
    assert np.array_equal(g.query_batch(pairs[:, 0], pairs[:, 1]), golden0[tag + "q_lca"])
