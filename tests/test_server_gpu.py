"""Query server with continuous batching (h2h_server_*): every request's
answers are the same when it runs alone and when it runs mixed with many
others (split over batches, sharing batches with other requests, several
batches in flight), and equal the direct batch API's; admission by memory,
out-of-range ids, removal and buffer checks."""
import threading

import numpy as np
import pytest

from conftest import sample13_files, write_multigraph

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graphs(tmp_path_factory):
    import gpuh2h
    root = str(tmp_path_factory.mktemp("serve"))
    p = gpuh2h.road_batch_params(1, 9000, 9000, seed=5)[0]
    gpuh2h.generate_road(root, "r", **p)
    specs = [(gpuh2h.files_for(root, "r"), p["partition_height"], 2), (write_multigraph(root), 6, 2),
             (sample13_files("Latitude"), 4, 1)]
    gs = []
    for f, H, C in specs:
        g = gpuh2h.Graph("s", H, C, 4, 1, files=f)
        g.contraction_noHub(1)
        g.constructLabel_noHub(2, 1, gpuh2h.LABEL_L4)
        gs.append(g)
    yield gs
    for g in gs:
        g.close()


def _requests(graphs, count, seed):
    import torch
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        gi = int(rng.integers(len(graphs)))
        n_v = graphs[gi].info()["n"]
        k = int(np.exp(rng.uniform(0, np.log(20000))))
        x = rng.integers(0, n_v, k).astype(np.int32)
        y = rng.integers(0, n_v, k).astype(np.int32)
        mode = int(rng.integers(2))
        if i % 3 == 0:  # page-locked buffers take the direct-transfer path
            xp = torch.from_numpy(x).pin_memory().numpy()
            yp = torch.from_numpy(y).pin_memory().numpy()
            reqs.append((gi, xp, yp, mode, True))
        else:
            reqs.append((gi, x, y, mode, False))
    return reqs


def _out(n, pinned):
    import torch
    if pinned:
        return torch.full((n,), -7, dtype=torch.int32).pin_memory().numpy()
    return np.full(n, -7, np.int32)


def test_alone_equals_mixed(graphs):
    import gpuh2h
    reqs = _requests(graphs, 80, 1)
    srv = gpuh2h.Server(slots=3, slot_pairs=6000)
    ids = [srv.add(g) for g in graphs]
    alone = []
    for gi, x, y, mode, pinned in reqs:
        out = _out(len(x), pinned)
        r = srv.submit(ids[gi], x, y, out, mode)
        srv.wait(r)
        srv.release(r)
        alone.append(out.copy())
        assert np.array_equal(out, graphs[gi].query(x, y, mode))
    srv.reset_stats()
    # the same requests all at once, from four threads
    outs = [_out(len(x), pinned) for gi, x, y, mode, pinned in reqs]
    rids = [None] * len(reqs)

    def sub(k):
        for j in range(k, len(reqs), 4):
            gi, x, y, mode, _ = reqs[j]
            rids[j] = srv.submit(ids[gi], x, y, outs[j], mode)
    th = [threading.Thread(target=sub, args=(k,)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    lats = []
    for j, r in enumerate(rids):
        srv.wait(r, 30_000_000)
        lats.append(srv.release(r))
        assert np.array_equal(outs[j], alone[j]), "request %d differs in the mix" % j
    st = srv.stats()
    assert st["requests"] == len(reqs) and st["pairs"] == sum(len(r[1]) for r in reqs)
    assert st["batches"] >= sum(len(r[1]) for r in reqs) // 6000
    assert st["max_inflight"] >= 2 and st["pending"] == 0
    assert min(lats) > 0
    srv.close()


def test_admission_ids_and_buffers(graphs):
    import gpuh2h
    small = gpuh2h.Server(slots=1, slot_pairs=1024, memory_budget=graphs[2].info()["device_bytes"] + 1)
    gid = small.add(graphs[2])
    with pytest.raises(gpuh2h.H2HError) as ex:
        small.add(graphs[0])
    assert ex.value.args[0].startswith("NOMEM")
    # out-of-range ids answer -1, the rest are exact
    x = np.array([0, 1, 99, -1, 5], np.int32)
    y = np.array([3, 1, 2, 4, 12], np.int32)
    out = np.zeros(5, np.int32)
    r = small.submit(gid, x, y, out)
    small.wait(r)
    small.release(r)
    ok = np.array([0, 1, 4], dtype=np.int64)
    assert out[2] == -1 and out[3] == -1
    assert np.array_equal(out[ok], graphs[2].query(x[ok], y[ok]))
    with pytest.raises(gpuh2h.H2HError):
        small.submit(gid + 5, x, y, out)
    small.remove(gid)
    with pytest.raises(gpuh2h.H2HError):
        small.submit(gid, x, y, out)
    assert small.add(graphs[2]) == 1        # the budget is free again
    # device buffers are refused
    import torch
    dx = torch.zeros(4, dtype=torch.int32, device="cuda")
    rid = gpuh2h.C.c_uint64()
    rc = small._L.h2h_server_submit(small.s, 1, dx.data_ptr(), dx.data_ptr(), dx.data_ptr(), 4, 0,
                                    gpuh2h.C.byref(rid))
    assert rc == -1
    small.close()
