"""The reference's own GPU code, executed: its partition-contraction kernel
(makeCHPerHeight_D_2, kernel_functions.cu:309-479), its GPU LL label fill
(makeH2HLabel_noCommunication_D_noHub_3 with the L4 father walk of
kernel_functions.cu:739-743 enabled) and its batched GPU query kernels, built
with nvcc for sm_103a from the reference's sources (oracle/build_ref_gpu.sh).

The golden fixtures come from the reference's CPU translation units, where
the GPU contraction kernel cannot run and the oracle's restatement of its
per-cell body stands in.  Here the real kernel runs, and every array it
leads to -- the elimination order, the contracted neighbour lists with their
shortcut weights, the tree, Euler tour, sparse table, labels and every query
answer -- must equal the fixtures: that executes the restated per-cell body
against the reference kernel on the 13-vertex sample (four partitions, every
ChangeToGlobalHeight) and the 64x64 grid (C = 1, 2, 6).

Runs where the reference sources were staged beside the oracle (they are
copied there from the reference tree by the build step); skipped elsewhere.
"""
import hashlib

import numpy as np
import pytest

from conftest import PARTS, sample13_files

pytestmark = pytest.mark.gpu

ARRAYS = ("order", "gpu_vertices", "father", "depth", "first", "rmq_hash", "rmq_id", "adj_hash", "adj_id", "adj_w",
          "dis_hash", "dis", "pos_hash", "pos_id", "pos_pos", "tree_bfs", "tree_hash", "q_lca", "q_nolca")


def _sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


@pytest.fixture(scope="module")
def ref_gpu():
    from oracle import oracle
    if not oracle.build_ref_gpu():
        pytest.skip("the reference's sources are not staged on this machine")
    return oracle


@pytest.mark.parametrize("meth,code,H", PARTS)
def test_reference_gpu_kernels_sample13(ref_gpu, golden13, meth, code, H):
    pairs = golden13["pairs13"]
    for C in range(1, H + 1):
        tag = "13_%s_C%d_L4/" % (meth, C)
        got = ref_gpu.run_reference(*sample13_files(meth), H, C, threads=2, l4=True, pairs=pairs, gpu=True)
        for k in ARRAYS:
            assert np.array_equal(got[k], golden13[tag + k]), (tag, k)


@pytest.mark.parametrize("C", [1, 2, 6])
def test_reference_gpu_kernels_cfg0(ref_gpu, cfg0_root, golden0, C):
    import gpuh2h
    tag = "cfg0_C%d_L4/" % C
    got = ref_gpu.run_reference(*gpuh2h.files_for(cfg0_root, "cfg0"), 6, C, threads=4, l4=True,
                                pairs=golden0["pairs"], gpu=True)
    for k in ("order", "father", "depth", "first", "tree_hash", "q_lca", "q_nolca", "gpu_vertices"):
        assert np.array_equal(got[k], golden0[tag + k]), k
    for k in ("rmq_hash", "rmq_id", "dis_hash", "dis", "pos_hash", "pos_id", "pos_pos", "tree_bfs", "adj_hash",
              "adj_id", "adj_w"):
        assert np.array_equal(_sha(got[k]), golden0[tag + "sha256/" + k]), k
    t = got["times"]
    assert t["queries"] == len(golden0["pairs"]) and t["H2HUsingTime_GPU"] >= 0
