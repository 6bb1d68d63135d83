import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "gpu-h2h_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")
SAMPLE13 = os.path.join(GOLDEN, "sample13")
PARTS = [("Latitude", 1, 4), ("Minimum", 2, 4), ("metis", 3, 3), ("scotch", 4, 3)]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def sample13_files(method_name):
    return (os.path.join(SAMPLE13, "Graph", "USA", "13Edge.txt"),
            os.path.join(SAMPLE13, "Partition", "13", method_name + "ID.txt"),
            os.path.join(SAMPLE13, "Partition", "13", method_name + "Cut.txt"))


@pytest.fixture(scope="session")
def golden13():
    return dict(np.load(os.path.join(GOLDEN, "sample13.npz")))


@pytest.fixture(scope="session")
def golden0():
    return dict(np.load(os.path.join(GOLDEN, "cfg0.npz")))


@pytest.fixture(scope="session")
def cfg0_root(tmp_path_factory):
    """The seeded 64x64 road-like grid (4,096 vertices, height-6 partition)."""
    import gpuh2h
    root = str(tmp_path_factory.mktemp("cfg0"))
    gpuh2h.generate_road(root, "cfg0")
    return root


def write_multigraph(root):
    """The 64x64 grid plus 200 parallel arc pairs (seeded): exercises the
    duplicate-merge and first-match rules of the elimination."""
    import shutil

    import gpuh2h
    gpuh2h.generate_road(root, "cfg0")
    e, i, c = gpuh2h.files_for(root, "cfg0")
    lines = open(e).read().split("\n")
    n = int(lines[0].split()[0])
    arcs = [l for l in lines[1:] if l.strip()]
    rng = np.random.default_rng(3)
    extra = []
    for k in rng.choice(len(arcs), 200, replace=False):
        _, u, v, w = arcs[k].split()
        w2 = max(1, int(w) + int(rng.integers(-3, 50)))
        extra += ["a %s %s %d" % (u, v, w2), "a %s %s %d" % (v, u, w2)]
    allarcs = arcs + extra
    os.makedirs(os.path.join(root, "Partition", "multi"), exist_ok=True)
    with open(os.path.join(root, "Graph", "USA", "multiEdge.txt"), "w") as f:
        f.write("%d %d\n" % (n, len(allarcs)) + "\n".join(allarcs) + "\n")
    shutil.copy(i, os.path.join(root, "Partition", "multi", "LatitudeID.txt"))
    shutil.copy(c, os.path.join(root, "Partition", "multi", "LatitudeCut.txt"))
    return gpuh2h.files_for(root, "multi")


@pytest.fixture(scope="session")
def multi_files(tmp_path_factory):
    return write_multigraph(str(tmp_path_factory.mktemp("multi")))
