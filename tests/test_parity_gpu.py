"""Parity of the CUDA path (through the C ABI) with the reference's outputs.

Golden fixtures come from the CPU build of the reference's own code
(tests/golden/make_golden.py); the elimination order, tree, Euler/RMQ table,
labels and every query answer must be identical (int32, zero tolerance).
"""
import hashlib

import numpy as np
import pytest

from conftest import PARTS, sample13_files

pytestmark = pytest.mark.gpu


def _sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def build(files, H, C, l4=True, pf=2, threads=4):
    import gpuh2h
    g = gpuh2h.Graph("t", H, C, threads, 1, files=files)
    g.contraction_noHub(1)
    g.constructLabel_noHub(pf, 1, gpuh2h.LABEL_L4 if l4 else gpuh2h.LABEL_L3)
    return g


def arrays(g):
    f, d, fi = g.tree()
    rh, ri = g.rmq()
    tb, th = g.bfs()
    return dict(order=g.order(), father=f, depth=d, first=fi, rmq_hash=rh, rmq_id=ri, tree_bfs=tb, tree_hash=th,
                **g.labels())


@pytest.mark.parametrize("meth,code,H", PARTS)
@pytest.mark.parametrize("l4", [True, False])
def test_sample13(golden13, meth, code, H, l4):
    import gpuh2h
    pairs = golden13["pairs13"]
    for C in range(1, H + 1):
        tag = "13_%s_C%d_%s/" % (meth, C, "L4" if l4 else "L3")
        g = build(sample13_files(meth), H, C, l4)
        got = arrays(g)
        for k, v in got.items():
            assert np.array_equal(v, golden13[tag + k]), (tag, k)
        assert np.array_equal(g.query(pairs[:, 0], pairs[:, 1], gpuh2h.QUERY_LCA), golden13[tag + "q_lca"])
        assert np.array_equal(g.query(pairs[:, 0], pairs[:, 1], gpuh2h.QUERY_NOLCA), golden13[tag + "q_nolca"])
        for a, b in pairs[::17]:
            assert g.H2HDistancQuery_UsingLCA_noHub(a, b) == golden13[tag + "q_lca"][a * 13 + b]
            assert g.H2HDistancQuery_noLCA_noHub(a, b) == golden13[tag + "q_nolca"][a * 13 + b]
        g.close()


@pytest.mark.parametrize("C", [1, 2, 6])
@pytest.mark.parametrize("l4", [True, False])
@pytest.mark.parametrize("pf", [2, 1])
def test_cfg0(cfg0_root, golden0, C, l4, pf):
    import gpuh2h
    tag = "cfg0_C%d_%s/" % (C, "L4" if l4 else "L3")
    g = build(gpuh2h.files_for(cfg0_root, "cfg0"), 6, C, l4, pf=pf)
    got = arrays(g)
    for k in ("order", "father", "depth", "first", "tree_hash"):
        assert np.array_equal(got[k], golden0[tag + k]), k
    for k in ("rmq_hash", "rmq_id", "dis_hash", "dis", "pos_hash", "pos_id", "pos_pos", "tree_bfs"):
        assert len(got[k]) == golden0[tag + "len/" + k][0], k
        if not np.array_equal(_sha(got[k]), golden0[tag + "sha256/" + k]):
            if k == "dis":
                s = golden0[tag + "dis_sample"]
                bad = np.nonzero(got["dis"][::97] != s)[0]
                pytest.fail("labels differ at %d sampled entries, first %s" % (len(bad), bad[:5] * 97))
            pytest.fail("array %s differs" % k)
    ah, aid, aw = g.adj()
    for k, v in (("adj_hash", ah), ("adj_id", aid), ("adj_w", aw)):
        assert np.array_equal(_sha(v), golden0[tag + "sha256/" + k]), k
    pairs = golden0["pairs"]
    assert np.array_equal(g.query(pairs[:, 0], pairs[:, 1], gpuh2h.QUERY_LCA), golden0[tag + "q_lca"])
    assert np.array_equal(g.query(pairs[:, 0], pairs[:, 1], gpuh2h.QUERY_NOLCA), golden0[tag + "q_nolca"])
    assert g.info()["gpu_vertices"] == golden0[tag + "gpu_vertices"][0]


@pytest.mark.parametrize("C", [1, 2])
def test_multigraph(multi_files, golden0, C):
    """Parallel arcs: duplicate merge at elimination and first-match fill-in."""
    import gpuh2h
    tag = "multi_C%d_L4/" % C
    g = build(multi_files, 6, C)
    assert np.array_equal(g.order(), golden0[tag + "order"])
    assert np.array_equal(g.tree()[0], golden0[tag + "father"])
    ah, aid, aw = g.adj()
    assert np.array_equal(_sha(aid), golden0[tag + "sha256/adj_id"])
    assert np.array_equal(_sha(aw), golden0[tag + "sha256/adj_w"])
    assert np.array_equal(_sha(g.labels()["dis"]), golden0[tag + "sha256/dis"])
    pairs = golden0["pairs"]
    assert np.array_equal(g.query(pairs[:, 0], pairs[:, 1], gpuh2h.QUERY_LCA), golden0[tag + "q_lca"])


def test_query_edge_cases(cfg0_root, golden0):
    import gpuh2h
    g = build(gpuh2h.files_for(cfg0_root, "cfg0"), 6, 1)
    # x == y answers 0 in both modes
    idx = np.arange(0, 4096, 7, dtype=np.int32)
    assert (g.query(idx, idx, gpuh2h.QUERY_LCA) == 0).all()
    assert (g.query(idx, idx, gpuh2h.QUERY_NOLCA) == 0).all()
    # empty batch
    assert len(g.query(np.empty(0, np.int32), np.empty(0, np.int32))) == 0
    # out-of-range vertex is an error, not a device fault
    with pytest.raises(gpuh2h.H2HError):
        g.query(np.array([0], np.int32), np.array([4096], np.int32))
    with pytest.raises(gpuh2h.H2HError):
        g.H2HDistancQuery_UsingLCA_noHub(-1, 3)
    # symmetric
    pairs = golden0["pairs"]
    a = g.query(pairs[:, 0], pairs[:, 1])
    b = g.query(pairs[:, 1], pairs[:, 0])
    assert np.array_equal(a, b)


def test_bad_device_batch_does_not_fail_later_host_calls(cfg0_root, golden0):
    """A device-buffer batch with an out-of-range id answers -1 for that pair;
    a clean host batch and a single-pair query on the same graph afterwards
    succeed (the host path has its own flag)."""
    import torch

    import gpuh2h
    g = build(gpuh2h.files_for(cfg0_root, "cfg0"), 6, 1)
    x = torch.tensor([0, 5, 9], dtype=torch.int32, device="cuda")
    y = torch.tensor([7, 4096, 3], dtype=torch.int32, device="cuda")
    out = torch.empty_like(x)
    g.query_device(x.data_ptr(), y.data_ptr(), out.data_ptr(), 3, gpuh2h.QUERY_LCA,
                   torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert out[1].item() == -1 and out[0].item() >= 0
    pairs = golden0["pairs"]
    tag = "cfg0_C1_L4/"
    assert np.array_equal(g.query(pairs[:, 0], pairs[:, 1], gpuh2h.QUERY_LCA), golden0[tag + "q_lca"])
    a, b = int(pairs[3, 0]), int(pairs[3, 1])
    assert g.H2HDistancQuery_UsingLCA_noHub(a, b) == golden0[tag + "q_lca"][3]
    # a bad host batch fails once, and the next clean one succeeds
    with pytest.raises(gpuh2h.H2HError):
        g.query(np.array([1], np.int32), np.array([-2], np.int32))
    assert np.array_equal(g.query(pairs[:, 0], pairs[:, 1], gpuh2h.QUERY_NOLCA), golden0[tag + "q_nolca"])
    g.close()


def test_device_batch_on_caller_stream(cfg0_root, golden0):
    import torch

    import gpuh2h
    g = build(gpuh2h.files_for(cfg0_root, "cfg0"), 6, 1)
    pairs = golden0["pairs"]
    x = torch.from_numpy(pairs[:, 0].copy()).cuda()
    y = torch.from_numpy(pairs[:, 1].copy()).cuda()
    out = torch.full_like(x, -7)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        g.H2HQuery_UsingLCA_noHub(x.data_ptr(), y.data_ptr(), out.data_ptr(), len(pairs), s.cuda_stream)
    s.synchronize()
    assert np.array_equal(out.cpu().numpy(), golden0["cfg0_C1_L4/q_lca"])
    g.H2HQuery_noLCA_noHub(x.data_ptr(), y.data_ptr(), out.data_ptr(), len(pairs), 0)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), golden0["cfg0_C1_L4/q_nolca"])


def test_unsupported_cpu_paths(cfg0_root):
    import gpuh2h
    g = gpuh2h.Graph("t", 6, 1, 2, 1, files=gpuh2h.files_for(cfg0_root, "cfg0"))
    with pytest.raises(gpuh2h.H2HError) as e:
        g.contraction_noHub(0)
    assert e.value.code == -7
    g.contraction_noHub(1)
    with pytest.raises(gpuh2h.H2HError) as e:
        g.constructLabel_noHub(2, 0)
    assert e.value.code == -7


def test_global_merge_staging(cfg0_root, golden0, monkeypatch):
    """The global-memory merge buffers that large separators use give the same result."""
    import gpuh2h
    monkeypatch.setenv("GPUH2H_GLOBAL_STAGING", "1")
    for C in (1, 2):
        tag = "cfg0_C%d_L4/" % C
        g = build(gpuh2h.files_for(cfg0_root, "cfg0"), 6, C)
        assert np.array_equal(g.order(), golden0[tag + "order"])
        assert np.array_equal(_sha(g.labels()["dis"]), golden0[tag + "sha256/dis"])


@pytest.mark.parametrize("envs", [{"GPUH2H_CLUSTER_HEAP": "1"}, {"GPUH2H_GRID_CELLS": "100000"},
                                  {"GPUH2H_GRID_CELLS": "100000", "GPUH2H_GRID_ARENA": "0"},
                                  {"GPUH2H_LEVEL_FILL": "1"}])
def test_alternate_kernels(cfg0_root, golden0, monkeypatch, envs):
    """Every elimination step on thread-block clusters (no cooperative
    launch), every step as one cooperative launch over all SMs (partition
    cells included) with merge buffers from the shared-memory arena or all
    in global memory, and the level-synchronous L4 fill (instead of the
    dataflow) give the same order, adjacency, labels and answers."""
    import gpuh2h
    for env, value in envs.items():
        monkeypatch.setenv(env, value)
    for C in (1, 2, 6):
        tag = "cfg0_C%d_L4/" % C
        g = build(gpuh2h.files_for(cfg0_root, "cfg0"), 6, C)
        assert np.array_equal(g.order(), golden0[tag + "order"])
        ah, aid, aw = g.adj()
        assert np.array_equal(_sha(aw), golden0[tag + "sha256/adj_w"])
        assert np.array_equal(_sha(g.labels()["dis"]), golden0[tag + "sha256/dis"])
        pairs = golden0["pairs"]
        assert np.array_equal(g.query(pairs[:, 0], pairs[:, 1], gpuh2h.QUERY_LCA), golden0[tag + "q_lca"])


@pytest.mark.parametrize("policy", [" ".join(["0/32/4"] * 12),
                                    "65536/64/32 65536/64/32 65536/64/32 0/64/32 "
                                    "262144/32/16 262144/32/16 262144/32/16 0/32/16 "
                                    "0/128/256 0/128/256 0/128/256 0/128/256"])
def test_tile_policies(cfg0_root, golden0, monkeypatch, policy):
    """Any tile shape of the dataflow fill gives the same labels."""
    import gpuh2h
    monkeypatch.setenv("GPUH2H_TILE_POLICY", policy)
    g = build(gpuh2h.files_for(cfg0_root, "cfg0"), 6, 2)
    assert np.array_equal(_sha(g.labels()["dis"]), golden0["cfg0_C2_L4/sha256/dis"])


@pytest.mark.parametrize("mapping", ["pair", "node"])
def test_plain_fill_baseline_matches(cfg0_root, mapping):
    """The reference's level-by-level fill mappings (the measurement
    baselines) reproduce the dataflow fill's labels exactly."""
    import gpuh2h
    for C in (1, 2):
        g = build(gpuh2h.files_for(cfg0_root, "cfg0"), 6, C)
        ms, bad = g.fill_labels_plain(mapping)
        assert bad == 0 and ms > 0
