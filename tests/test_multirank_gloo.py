"""bench.py's multi-rank host logic on two gloo ranks (CPU): each replica draws
its own query batch, barriers bracket the timed region and the reported time is
the maximum over ranks.  No GPU and no collective on the data path."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (repo, os.path.join(repo, "gpu-h2h_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist

    import bench
    import gpuh2h
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_setup() == (world, rank, rank)
    x, y = gpuh2h.uniform_pairs(4096, 1000, bench.rank_query_seed(rank))
    bench.barrier(world)
    t_max = bench.reduce_max(float(rank + 1) * 0.5, world)
    np.save(os.path.join(out_dir, "r%d.npy" % rank), np.concatenate([x[:10], y[:10]]))
    with open(os.path.join(out_dir, "t%d.txt" % rank), "w") as f:
        f.write(repr(t_max))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    a, b = np.load(tmp_path / "r0.npy"), np.load(tmp_path / "r1.npy")
    assert not np.array_equal(a, b), "replicas must draw different query batches"
    assert float(open(tmp_path / "t0.txt").read()) == 1.0
    assert float(open(tmp_path / "t1.txt").read()) == 1.0
