"""Batched construction (h2h_batch_*): every graph of a mixed batch must
equal its own single-graph build bit for bit (elimination order, tree, Euler
/ sparse table, shortcut lists, labels, query answers); a rebuild after new
weights must equal a fresh build from an Edge file holding those weights;
tuning the fill's tile shapes must not change a label."""
import os
import shutil

import numpy as np
import pytest

from conftest import sample13_files, write_multigraph

pytestmark = pytest.mark.gpu


def _single(files, H, C):
    import gpuh2h
    g = gpuh2h.Graph("s", H, C, 4, 1, files=files)
    g.contraction_noHub(1)
    g.constructLabel_noHub(2, 1, gpuh2h.LABEL_L4)
    return g


def _arrays(g):
    f, d, fi = g.tree()
    rh, ri = g.rmq()
    tb, th = g.bfs()
    ah, aid, aw = g.adj()
    return dict(order=g.order(), father=f, depth=d, first=fi, rmq_hash=rh, rmq_id=ri, tree_bfs=tb, tree_hash=th,
                adj_hash=ah, adj_id=aid, adj_w=aw, **g.labels())


def _same(a, b, tag):
    for k in a:
        assert np.array_equal(a[k], b[k]), "%s: %s differs" % (tag, k)


def _queries(g, n, seed):
    import gpuh2h
    x, y = gpuh2h.uniform_pairs(n, 4000, seed)
    return x, y, g.query(x, y, gpuh2h.QUERY_LCA)


@pytest.fixture(scope="module")
def batch_specs(tmp_path_factory):
    """(files, H, C) of a mixed batch: six seeded road graphs of 2k-12k
    vertices, the 13-vertex sample, the 4,096-vertex grid with parallel arcs,
    and the grid again with every level global (H == C)."""
    import gpuh2h
    root = str(tmp_path_factory.mktemp("batch"))
    specs = []
    for i, p in enumerate(gpuh2h.road_batch_params(6, 2000, 12000, seed=11)):
        name = "b%d" % i
        gpuh2h.generate_road(root, name, **p)
        specs.append((gpuh2h.files_for(root, name), p["partition_height"], 2))
    specs.append((sample13_files("Latitude"), 4, 1))
    specs.append((write_multigraph(root), 6, 2))
    specs.append((gpuh2h.files_for(root, "cfg0"), 6, 6))
    return root, specs


@pytest.mark.parametrize("grid_cells", [None, "0", "100000"])
def test_batch_matches_single_builds(batch_specs, monkeypatch, grid_cells):
    """Default launch shapes; every step on clusters; every step (all graphs'
    cells, global orders included) as one cooperative launch."""
    import gpuh2h
    if grid_cells is not None:
        monkeypatch.setenv("GPUH2H_GRID_CELLS", grid_cells)
    _, specs = batch_specs
    graphs = [gpuh2h.Graph("b", H, C, 4, 1, files=f) for f, H, C in specs]
    b = gpuh2h.Batch(graphs, threads=4)
    inf = b.info()
    assert inf["graphs"] == len(specs) and inf["vertices"] == sum(g.info()["n"] for g in graphs)
    assert inf["elim_launches"] >= 1 and inf["fill_tiles"] >= inf["vertices"]
    for (f, H, C), g in zip(specs, graphs):
        s = _single(f, H, C)
        _same(_arrays(s), _arrays(g), "graph %s H=%d C=%d" % (os.path.basename(f[0]), H, C))
        n = g.info()["n"]
        x, y, r = _queries(g, n, 5)
        assert np.array_equal(r, s.query(x, y, gpuh2h.QUERY_LCA))
        assert np.array_equal(r, g.query(x, y, gpuh2h.QUERY_NOLCA))
        assert g.info()["max_label"] == s.info()["max_label"]
        s.close()
    b.close()
    for g in graphs:
        g.close()


def test_rebuild_with_new_weights_equals_fresh_build(batch_specs, tmp_path):
    import gpuh2h
    _, specs = batch_specs
    graphs = [gpuh2h.Graph("b", H, C, 4, 1, files=f) for f, H, C in specs]
    b = gpuh2h.Batch(graphs, threads=4)
    before = [g.labels()["dis"] for g in graphs]
    b.rebuild()                       # same weights: same labels, now through the captured graph
    inf = b.info()
    assert inf["graph_captured"] == 1
    assert 0 < inf["t_rebuild_fill_us"] <= inf["t_rebuild_us"]
    for g, d in zip(graphs, before):
        assert np.array_equal(g.labels()["dis"], d)
    # symmetric new weights for three graphs
    changed = {0: None, len(specs) - 2: None, len(specs) - 3: None}
    for gi in changed:
        off, v, w = graphs[gi].input_arcs()
        n = len(off) - 1
        src = np.repeat(np.arange(n), np.diff(off))
        lo, hi = np.minimum(src, v).astype(np.int64), np.maximum(src, v).astype(np.int64)
        w2 = (w.astype(np.int64) + (lo * 31 + hi * 17) % 97 + 1).astype(np.int32)
        changed[gi] = w2
        b.set_weights(gi, w2)
    b.rebuild()
    b.sync_host()
    for gi, (f, H, C) in enumerate(specs):
        g = graphs[gi]
        if gi in changed:
            d = tmp_path / ("w%d" % gi)
            os.makedirs(d)
            off, v, _ = g.input_arcs()
            edge = str(d / "Edge.txt")
            gpuh2h.write_edge_file(edge, off, v, changed[gi])
            s = _single((edge, f[1], f[2]), H, C)
        else:
            s = _single(f, H, C)
        _same(_arrays(s), _arrays(g), "graph %d after rebuild" % gi)
        x, y, r = _queries(g, g.info()["n"], 9)
        assert np.array_equal(r, s.query(x, y, gpuh2h.QUERY_LCA))
        s.close()
    b.close()
    for g in graphs:
        g.close()


def test_tuned_policy_keeps_labels(batch_specs):
    import gpuh2h
    _, specs = batch_specs
    graphs = [gpuh2h.Graph("b", H, C, 4, 1, files=f) for f, H, C in specs[:4]]
    b = gpuh2h.Batch(graphs, threads=4)
    ref = [g.labels()["dis"] for g in graphs]
    default = b.policy()
    pol = b.tune(1)
    assert pol == b.policy() and len(pol.split()) == 12
    for g, d in zip(graphs, ref):
        assert np.array_equal(g.labels()["dis"], d)
    # a hand-set policy that splits every node finely
    b.set_policy(" ".join(["0/32/8"] * 12))
    b.rebuild()
    for g, d in zip(graphs, ref):
        assert np.array_equal(g.labels()["dis"], d)
    b.set_policy(default)
    with pytest.raises(gpuh2h.H2HError):
        b.set_policy("1/2/3")
    b.close()
    for g in graphs:
        g.close()


def test_batch_state_errors(batch_specs):
    import gpuh2h
    _, specs = batch_specs
    f, H, C = specs[0]
    g = gpuh2h.Graph("b", H, C, 4, 1, files=f)
    g.contraction_noHub(1)
    with pytest.raises(gpuh2h.H2HError) as ex:
        gpuh2h.Batch([g])
    assert ex.value.args[0].startswith("STATE")
    g2 = gpuh2h.Graph("b", H, C, 4, 1, files=f)
    with pytest.raises(gpuh2h.H2HError):
        gpuh2h.Batch([g2, g2])
    b = gpuh2h.Batch([g2])
    with pytest.raises(gpuh2h.H2HError):
        b.set_weights(3, np.zeros(10, np.int32))
    with pytest.raises(gpuh2h.H2HError):
        g2.contraction_noHub(1)     # already built by the batch
    b.close()
    g.close()
    g2.close()
