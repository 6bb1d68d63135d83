"""The built index on disk: a handle read back with h2h_load_index answers
every query and serves every accessor exactly like the handle that was
saved (single build and a batch graph) and like the reference's golden
outputs for the same graph; a damaged file is refused."""
import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _all(g):
    f, d, fi = g.tree()
    rh, ri = g.rmq()
    tb, th = g.bfs()
    ah, aid, aw = g.adj()
    return dict(order=g.order(), father=f, depth=d, first=fi, rmq_hash=rh, rmq_id=ri, tree_bfs=tb, tree_hash=th,
                adj_hash=ah, adj_id=aid, adj_w=aw, **g.labels())


def _check_same(a, b, tmp_path):
    import gpuh2h
    A, B = _all(a), _all(b)
    for k in A:
        assert np.array_equal(A[k], B[k]), k
    n = a.info()["n"]
    x, y = gpuh2h.uniform_pairs(n, 20000, 3)
    for mode in (gpuh2h.QUERY_LCA, gpuh2h.QUERY_NOLCA):
        assert np.array_equal(a.query(x, y, mode), b.query(x, y, mode))
    ia, ib = a.info(), b.info()
    for k in ("n", "head", "tree_height", "label_size", "pos_size", "rmq_size", "euler_size", "adj_size",
              "max_label", "label_mode", "gpu_vertices"):
        assert ia[k] == ib[k], k


def _sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def _check_golden(h, golden0, tag):
    """The loaded handle against the reference's own outputs (C = 2, L4)."""
    import gpuh2h
    A = _all(h)
    for k in ("order", "father", "depth", "first", "tree_hash"):
        assert np.array_equal(A[k], golden0[tag + k]), k
    for k in ("rmq_hash", "rmq_id", "dis_hash", "dis", "pos_hash", "pos_id", "pos_pos", "tree_bfs", "adj_hash",
              "adj_id", "adj_w"):
        assert np.array_equal(_sha(A[k]), golden0[tag + "sha256/" + k]), k
    pairs = golden0["pairs"]
    assert np.array_equal(h.query(pairs[:, 0], pairs[:, 1], gpuh2h.QUERY_LCA), golden0[tag + "q_lca"])
    assert np.array_equal(h.query(pairs[:, 0], pairs[:, 1], gpuh2h.QUERY_NOLCA), golden0[tag + "q_nolca"])


def test_save_load_single(cfg0_root, golden0, tmp_path):
    import gpuh2h
    g = gpuh2h.Graph("cfg0", 6, 2, 4, 1, files=gpuh2h.files_for(cfg0_root, "cfg0"))
    g.contraction_noHub(1).constructLabel_noHub(2, 1, gpuh2h.LABEL_L4)
    p = str(tmp_path / "cfg0.idx")
    g.save_index(p)
    h = gpuh2h.Graph.load_index(p)
    _check_same(g, h, tmp_path)
    _check_golden(h, golden0, "cfg0_C2_L4/")
    with pytest.raises(gpuh2h.H2HError):
        h.local_pairs(10)                 # no input arcs in a loaded index
    # a damaged position list is refused
    raw = bytearray(open(p, "rb").read())
    i = g.info()
    pos_pos_at = len(raw) - (i["label_size"] * 4 + 16) - (i["n"] * 4 + 16) - ((i["n_levels"] + 1) * 4 + 16) - \
        i["pos_size"] * 4
    raw[pos_pos_at:pos_pos_at + 4] = (10 ** 6).to_bytes(4, "little")
    bad = tmp_path / "bad.idx"
    bad.write_bytes(bytes(raw))
    with pytest.raises(gpuh2h.H2HError) as ex:
        gpuh2h.Graph.load_index(str(bad))
    assert ex.value.args[0].startswith("FORMAT")
    g.close()
    h.close()


def test_save_load_batch_graph(cfg0_root, golden0, tmp_path):
    import gpuh2h
    from conftest import sample13_files
    gs = [gpuh2h.Graph("s", 4, 1, 2, 1, files=sample13_files("Latitude")),
          gpuh2h.Graph("cfg0", 6, 2, 4, 1, files=gpuh2h.files_for(cfg0_root, "cfg0"))]
    b = gpuh2h.Batch(gs, threads=2)
    p = str(tmp_path / "b.idx")
    gs[1].save_index(p)
    h = gpuh2h.Graph.load_index(p)
    _check_same(gs[1], h, tmp_path)
    _check_golden(h, golden0, "cfg0_C2_L4/")
    h.close()
    b.close()
    for g in gs:
        g.close()
