"""The allocation-free L4 label fill, h2h_fill_labels_l4_noalloc, through the C ABI.

Some callers cannot call cudaMalloc -- code that runs inside another
framework's device-memory budget, or a plugin that may only use the buffers
its host hands it.  For them the library offers one entry point whose
scratch lives in a fixed on-device array; the caller passes inputs and the
output.  This test hands it the tree of an index built by the regular path
and checks, on two calls in a row, that it writes exactly the labels the
regular path wrote and the reference's golden labels (int32, zero
tolerance), and that malformed inputs are refused before anything is
written.  The file name sorts last so
a run that stops at the first failure has already run every other test.
"""
import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(g):
    father, depth, _ = g.tree()
    order, _ = g.bfs()
    lab = g.labels()
    ah, aid, aw = g.adj()
    n = len(father)
    ph = lab["pos_hash"]
    owner = np.repeat(np.arange(n, dtype=np.int64), np.diff(ph))
    adj_owner = np.repeat(np.arange(n, dtype=np.int64), np.diff(ah))
    key_adj = adj_owner * n + aid
    key_pos = owner * n + lab["pos_id"]
    idx = np.minimum(np.searchsorted(key_adj, key_pos), max(len(key_adj) - 1, 0))
    pos_w = np.where(lab["pos_id"] == owner, 0, aw[idx]).astype(np.int32)
    assert np.array_equal(np.where(lab["pos_id"] == owner, key_pos, key_adj[idx]), key_pos)
    return dict(order=order, father=father, depth=depth, pos_hash=ph, pos_id=lab["pos_id"], pos_pos=lab["pos_pos"],
                pos_w=pos_w, dis_hash=lab["dis_hash"]), lab["dis"]


def _sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def test_noalloc_fill_matches_regular_path_twice(cfg0_root, golden0):
    import torch

    import gpuh2h
    g = gpuh2h.Graph("t", 6, 1, 4, 1, files=gpuh2h.files_for(cfg0_root, "cfg0"))
    g.contraction_noHub(1)
    g.constructLabel_noHub(2, 1, gpuh2h.LABEL_L4)
    host, expected = _inputs(g)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in host.items()}
    n = len(host["father"])
    total = int(host["dis_hash"][-1])
    max_depth = int(host["depth"].max())
    max_sep = int((np.diff(host["pos_hash"]) - 1).max())
    out = torch.full((total,), -7, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream()
    for call in range(2):
        out.fill_(-7)
        gpuh2h.fill_labels_l4_noalloc(n, dev["order"].data_ptr(), dev["father"].data_ptr(), dev["depth"].data_ptr(),
                                      dev["pos_hash"].data_ptr(), dev["pos_id"].data_ptr(),
                                      dev["pos_pos"].data_ptr(), dev["pos_w"].data_ptr(),
                                      dev["dis_hash"].data_ptr(), total, out.data_ptr(), max_depth, max_sep,
                                      s.cuda_stream)
        got = out.cpu().numpy()
        bad = np.nonzero(got != expected)[0]
        assert len(bad) == 0, "call %d: %d label entries differ, first at %s" % (call, len(bad), bad[:5])
        # the reference's own L4 labels for this graph and partition (C = 1)
        assert len(got) == golden0["cfg0_C1_L4/len/dis"][0]
        assert np.array_equal(_sha(got), golden0["cfg0_C1_L4/sha256/dis"]), "call %d: differs from the golden" % call
    # a tree beyond the fixed scratch is refused before any device work
    with pytest.raises(gpuh2h.H2HError) as e:
        gpuh2h.fill_labels_l4_noalloc(n, dev["order"].data_ptr(), dev["father"].data_ptr(), dev["depth"].data_ptr(),
                                      dev["pos_hash"].data_ptr(), dev["pos_id"].data_ptr(),
                                      dev["pos_pos"].data_ptr(), dev["pos_w"].data_ptr(),
                                      dev["dis_hash"].data_ptr(), 1 << 23, out.data_ptr(), max_depth, max_sep,
                                      s.cuda_stream)
    assert e.value.code == -1


def test_noalloc_fill_wait_runs_out_then_recovers(cfg0_root):
    """A dependency that never completes ends the fill with an error status
    instead of a hang: the order below drops the root (its children wait for
    a flag that nothing sets) and every wait is bounded (about 2 s), so the
    kernel returns H2H_ERR_DEVICE; the context stays usable and the next call,
    with the proper order, writes the regular path's labels."""
    import torch

    import gpuh2h
    g = gpuh2h.Graph("t", 6, 1, 4, 1, files=gpuh2h.files_for(cfg0_root, "cfg0"))
    g.contraction_noHub(1)
    g.constructLabel_noHub(2, 1, gpuh2h.LABEL_L4)
    host, expected = _inputs(g)
    broken = host["order"].copy()
    assert host["father"][broken[0]] < 0  # the level order starts at the root
    broken[0] = broken[1]                 # the root is never filled
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in host.items()}
    d_broken = torch.from_numpy(np.ascontiguousarray(broken)).cuda()
    n = len(host["father"])
    total = int(host["dis_hash"][-1])
    max_depth = int(host["depth"].max())
    max_sep = int((np.diff(host["pos_hash"]) - 1).max())
    out = torch.full((total,), -7, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream()

    def run(order):
        gpuh2h.fill_labels_l4_noalloc(n, order.data_ptr(), dev["father"].data_ptr(), dev["depth"].data_ptr(),
                                      dev["pos_hash"].data_ptr(), dev["pos_id"].data_ptr(),
                                      dev["pos_pos"].data_ptr(), dev["pos_w"].data_ptr(),
                                      dev["dis_hash"].data_ptr(), total, out.data_ptr(), max_depth, max_sep,
                                      s.cuda_stream)

    with pytest.raises(gpuh2h.H2HError) as e:
        run(d_broken)
    assert e.value.code == -8 and "wait ran out" in str(e.value)
    out.fill_(-7)
    run(dev["order"])
    assert np.array_equal(out.cpu().numpy(), expected)


@pytest.mark.parametrize("case", ["depth_zero", "dis_hash_not_monotone", "father_wrong_level", "father_out_of_range",
                                  "pos_id_out_of_range", "pos_list_unsorted"])
def test_noalloc_fill_rejects_malformed_inputs(cfg0_root, case):
    """Each malformed input is refused by the validation pass with nothing
    written: the output buffer, padded with guard entries on both sides,
    keeps its fill value everywhere.  Every input buffer is also padded, so
    the inputs stay inside their allocations whatever is read."""
    import torch

    import gpuh2h
    g = gpuh2h.Graph("t", 6, 1, 4, 1, files=gpuh2h.files_for(cfg0_root, "cfg0"))
    g.contraction_noHub(1)
    g.constructLabel_noHub(2, 1, gpuh2h.LABEL_L4)
    host, _ = _inputs(g)
    host = {k: v.copy() for k, v in host.items()}
    n = len(host["father"])
    leaf = int(np.nonzero(host["depth"] == host["depth"].max())[0][0])
    mid = int(np.nonzero(host["depth"] > 3)[0][0])
    if case == "depth_zero":
        host["depth"][leaf] = 0
    elif case == "dis_hash_not_monotone":
        host["dis_hash"][n // 2] = host["dis_hash"][n // 2 + 1] + 1
    elif case == "father_wrong_level":
        host["father"][mid] = host["father"][host["father"][mid]]
    elif case == "father_out_of_range":
        host["father"][mid] = n
    elif case == "pos_id_out_of_range":
        host["pos_id"][host["pos_hash"][mid]] = n + 5
    elif case == "pos_list_unsorted":
        a = host["pos_hash"][mid]
        host["pos_pos"][a], host["pos_pos"][a + 1] = host["pos_pos"][a + 1], host["pos_pos"][a]
    pad = 64
    dev = {}
    for k, v in host.items():
        buf = torch.zeros(len(v) + 2 * pad, dtype=torch.int64 if v.dtype == np.int64 else torch.int32,
                          device="cuda")
        buf[pad:pad + len(v)] = torch.from_numpy(np.ascontiguousarray(v)).cuda()
        dev[k] = buf
    total = int(host["dis_hash"][-1])
    max_depth = int(host["depth"].max())
    max_sep = int((np.diff(host["pos_hash"]) - 1).max())
    out = torch.full((total + 2 * pad,), -7, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream()
    ptr = lambda k: dev[k].data_ptr() + pad * dev[k].element_size()
    with pytest.raises(gpuh2h.H2HError) as e:
        gpuh2h.fill_labels_l4_noalloc(n, ptr("order"), ptr("father"), ptr("depth"), ptr("pos_hash"), ptr("pos_id"),
                                      ptr("pos_pos"), ptr("pos_w"), ptr("dis_hash"), total,
                                      out.data_ptr() + pad * 4, max_depth, max_sep, s.cuda_stream)
    assert e.value.code == -8 and "rejected before any write" in str(e.value)
    assert bool((out == -7).all()), "a rejected call wrote to the output"
