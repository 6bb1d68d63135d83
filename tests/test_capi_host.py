"""C-ABI checks that need no GPU: exported symbols, loader validation and
error codes, state errors before a build, the workload generators and the
G2H argument-count rule (Graph_Fundamental.cu:4-95, main.cu:244-247)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import REPO, sample13_files


def _declared():
    names = set()
    for f in os.listdir(os.path.join(REPO, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(REPO, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(h2h_\w+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    import gpuh2h
    L = gpuh2h.load_library()
    declared = _declared()
    assert len(declared) >= 25
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, missing
    # the Python mirror binds every declared entry point with a signature
    assert declared <= set(gpuh2h.SIGNATURES), sorted(declared - set(gpuh2h.SIGNATURES))


def _load(files, H=4, Cg=1, threads=2):
    import gpuh2h
    L = gpuh2h.load_library()
    h = C.c_void_p()
    rc = L.h2h_load_files(*[f.encode() for f in files], b"t", H, Cg, threads, 1, C.byref(h))
    return rc, h


def test_load_sample_and_state_errors():
    import gpuh2h
    L = gpuh2h.load_library()
    rc, h = _load(sample13_files("Latitude"))
    assert rc == 0 and h
    info = gpuh2h._Info()
    assert L.h2h_get_info(h, C.byref(info)) == 0
    assert info.n == 13 and info.m == 44 and info.partition_height == 4
    # accessors before h2h_contract / h2h_build_labels report a state error
    a = np.empty(13, np.int32)
    assert L.h2h_copy_order(h, gpuh2h._p(a)) == -4
    assert L.h2h_copy_labels(h, None, None, None, None, None) == -4
    assert L.h2h_query_lca_nohub(h, 0, 1) == -1
    assert b"labels not built" in L.h2h_last_error()
    # the CPU alternatives of the reference are outside the GPU hot path
    assert L.h2h_contract(h, 0) == -7
    assert L.h2h_build_labels(h, 2, 1, 4) == -4
    L.h2h_free(h)


def test_load_paths_follow_g2h_rules(tmp_path):
    import shutil

    import gpuh2h
    root = str(tmp_path)
    os.makedirs(os.path.join(root, "Graph", "USA"))
    os.makedirs(os.path.join(root, "Partition", "13"))
    e, i, c = sample13_files("metis")
    shutil.copy(e, os.path.join(root, "Graph", "USA", "13Edge.txt"))
    shutil.copy(i, os.path.join(root, "Partition", "13", "metisID.txt"))
    shutil.copy(c, os.path.join(root, "Partition", "13", "metisCut.txt"))
    g = gpuh2h.Graph("13", 3, 1, 2, 3, root=root)          # method 3 = metis
    assert g.info()["n"] == 13
    with pytest.raises(gpuh2h.H2HError) as ex:
        gpuh2h.Graph("13", 3, 1, 2, 1, root=root)          # Latitude files are absent
    assert ex.value.code == -2


def _write(path, text):
    with open(path, "w") as f:
        f.write(text)


@pytest.mark.parametrize("case,code", [
    ("truncated_edge", -3), ("bad_vertex", -3), ("count_mismatch", -3), ("cut_rows", -3), ("asymmetric", -7),
    ("disconnected", -7), ("change_height", -1), ("zero_change", -1)])
def test_loader_rejects_bad_input(tmp_path, case, code):
    e, i, c = sample13_files("Latitude")
    edge, idf, cut = (open(p).read() for p in (e, i, c))
    H, Cg = 4, 1
    if case == "truncated_edge":
        edge = "\n".join(edge.split("\n")[:20])
    elif case == "bad_vertex":
        edge = edge.replace("a 1 2 4", "a 1 99 4", 1)
    elif case == "count_mismatch":
        edge = edge.replace("13 44", "14 44", 1)
    elif case == "cut_rows":
        cut = "\n".join(cut.split("\n")[:5])
    elif case == "asymmetric":
        lines = edge.strip().split("\n")
        lines = [l for l in lines[1:] if l.strip() != "a 2 1 4"]
        edge = "13 %d\n" % len(lines) + "\n".join(lines) + "\n"
    elif case == "disconnected":
        lines = [l for l in edge.strip().split("\n")[1:] if not (l.split()[1] in ("13",) or l.split()[2] in ("13",))]
        edge = "13 %d\n" % len(lines) + "\n".join(lines) + "\n"
    elif case == "change_height":
        Cg = 5
    elif case == "zero_change":
        Cg = 0
    paths = []
    for name, text in (("E.txt", edge), ("I.txt", idf), ("C.txt", cut)):
        p = str(tmp_path / name)
        _write(p, text)
        paths.append(p)
    rc, h = _load(paths, H, Cg)
    assert rc == code
    assert not h


def test_missing_file_is_io_error(tmp_path):
    rc, h = _load([str(tmp_path / "nope.txt")] * 3)
    assert rc == -2


def test_generators_are_seeded_and_in_range(cfg0_root):
    import gpuh2h
    x1, y1 = gpuh2h.uniform_pairs(4096, 1000, 9)
    x2, y2 = gpuh2h.uniform_pairs(4096, 1000, 9)
    assert np.array_equal(x1, x2) and np.array_equal(y1, y2)
    assert x1.min() >= 0 and x1.max() < 4096
    g = gpuh2h.Graph("cfg0", 6, 1, 2, 1, files=gpuh2h.files_for(cfg0_root, "cfg0"))
    lx, ly = g.local_pairs(500, 20, 3)
    assert lx.min() >= 0 and ly.max() < 4096
    # t is reachable from s within 20 hops
    e = gpuh2h.files_for(cfg0_root, "cfg0")[0]
    arcs = np.loadtxt(e, skiprows=1, usecols=(1, 2), dtype=np.int64) - 1
    adj = [[] for _ in range(4096)]
    for a, b in arcs:
        adj[a].append(b)
    for s, t in zip(lx[:50], ly[:50]):
        seen, frontier = {int(s)}, [int(s)]
        for _ in range(20):
            frontier = [w for v in frontier for w in adj[v] if w not in seen]
            seen.update(frontier)
        assert int(t) in seen


def test_oracle_generators_equal_library_generators(tmp_path):
    """The CPU baseline draws its graph and pairs through the oracle library
    (no GPU library in that process): same files, same uniform and local
    pairs as the library's generators."""
    import gpuh2h
    from oracle import oracle
    kw = dict(n=20000, target_arcs=55000, aspect_milli=1300, jitter_milli=300, diag_permille=50, hw_tiers=2,
              hw_permille10=50, hw_k=3, hw_scale_milli=400, partition_height=7, seed=11, cols=0, drop_permille=0)
    a, b = str(tmp_path / "lib"), str(tmp_path / "ora")
    assert gpuh2h.generate_road(a, "w", **kw) == oracle.generate_road(b, "w", **kw)
    for fa, fb in zip(gpuh2h.files_for(a, "w"), gpuh2h.files_for(b, "w")):
        assert open(fa, "rb").read() == open(fb, "rb").read(), fa
    for u, v in zip(gpuh2h.uniform_pairs(20000, 5000, 3), oracle.uniform_pairs(20000, 5000, 3)):
        assert np.array_equal(u, v)
    files = gpuh2h.files_for(a, "w")
    g = gpuh2h.Graph("w", 7, 2, 2, 1, files=files)
    o = oracle.OracleGraph(*files, 7, 2, 2)
    for u, v in zip(g.local_pairs(5000, 20, 5), o.local_pairs(5000, 20, 5)):
        assert np.array_equal(u, v)
    off, v, _ = g.input_arcs()
    off2, v2 = o.input_arcs()
    assert np.array_equal(off, off2) and np.array_equal(v, v2)
    g.close()
    o.close()


def test_loader_keeps_file_order_for_ungrouped_arcs(tmp_path):
    """adjList is push_back in file order (Graph_Fundamental.cu:46-55): an Edge
    file whose arcs are not grouped by tail loads into the same lists as a
    plain stable grouping of its lines, with self loops dropped."""
    import shutil

    import gpuh2h
    root = str(tmp_path)
    gpuh2h.generate_road(root, "cfg0")
    e, i, c = gpuh2h.files_for(root, "cfg0")
    lines = open(e).read().split("\n")
    n, m = map(int, lines[0].split())
    arcs = [l for l in lines[1:] if l.strip()]
    rng = np.random.default_rng(5)
    arcs = [arcs[k] for k in rng.permutation(len(arcs))] + ["a 7 7 5"]  # plus a self loop
    os.makedirs(os.path.join(root, "Partition", "shuf"), exist_ok=True)
    with open(os.path.join(root, "Graph", "USA", "shufEdge.txt"), "w") as f:
        f.write("%d %d\n" % (n, len(arcs)) + "\n".join(arcs) + "\n")
    shutil.copy(i, os.path.join(root, "Partition", "shuf", "LatitudeID.txt"))
    shutil.copy(c, os.path.join(root, "Partition", "shuf", "LatitudeCut.txt"))
    g = gpuh2h.Graph("shuf", 6, 1, 4, 1, files=gpuh2h.files_for(root, "shuf"))
    off, v, w = g.input_arcs()
    lists = [[] for _ in range(n)]
    for l in arcs:
        _, a, b, ww = l.split()
        if a != b:
            lists[int(a) - 1].append((int(b) - 1, int(ww)))
    assert off[-1] == sum(len(x) for x in lists)
    for u in range(0, n, 37):
        got = list(zip(v[off[u]:off[u + 1]].tolist(), w[off[u]:off[u + 1]].tolist()))
        assert got == lists[u], u
    g.close()


def test_g2h_cli_argument_count_rule(tmp_path):
    from gpuh2h import _build
    _build.build()
    for argv in ([], ["13"], ["13", "4", "1", "2", "1", "1", "2"]):
        r = subprocess.run([_build.CLI] + argv, cwd=str(tmp_path), capture_output=True, timeout=60)
        assert r.returncode == 0 and r.stdout == b"" and r.stderr == b""


def test_index_file_validation(tmp_path):
    """h2h_load_index rejects missing, foreign and truncated files before it
    touches a GPU."""
    import gpuh2h
    L = gpuh2h.load_library()
    h = C.c_void_p()
    assert L.h2h_load_index(str(tmp_path / "none.idx").encode(), C.byref(h)) == -2
    bad = tmp_path / "bad.idx"
    bad.write_bytes(b"NOTANIDX" + b"\0" * 64)
    assert L.h2h_load_index(str(bad).encode(), C.byref(h)) == -3
    trunc = tmp_path / "trunc.idx"
    trunc.write_bytes(b"GPUH2HIX" + (1).to_bytes(4, "little") + (16).to_bytes(4, "little") + b"\0" * 10)
    assert L.h2h_load_index(str(trunc).encode(), C.byref(h)) == -3
    # a header whose counts disagree (n = 5, euler_n = 3)
    import struct
    hdr = struct.pack("<9q8i", 5, 8, 3, 10, 4, 9, 15, 7, 9, 3, 1, 4, 0, 3, 5, 1, 3)
    incons = tmp_path / "incons.idx"
    incons.write_bytes(b"GPUH2HIX" + struct.pack("<II", 1, 16) + hdr + struct.pack("<I", 0))
    assert L.h2h_load_index(str(incons).encode(), C.byref(h)) == -3
    assert not h


def test_parallel_loader_equals_serial(tmp_path):
    """Files big enough for the chunked parsers (over 1 MB: 60k vertices)
    load to exactly what the one-token-at-a-time reader gives: partition
    array, CSR arcs in file order.  A file whose records break the one-per-line
    layout falls back to the token reader and still loads the same; a
    duplicated ID record is rejected either way."""
    import gpuh2h
    root = str(tmp_path)
    gpuh2h.generate_road(root, "p", n=60000, target_arcs=170000, aspect_milli=1300, jitter_milli=300,
                         diag_permille=50, hw_tiers=1, hw_permille10=50, hw_k=3, hw_scale_milli=400,
                         partition_height=8, seed=5, cols=0, drop_permille=0)
    files = gpuh2h.files_for(root, "p")
    assert os.path.getsize(files[0]) > (1 << 20) and os.path.getsize(files[1]) > (1 << 20)

    def load(fs, threads):
        g = gpuh2h.Graph("p", 8, 2, threads, 1, files=fs)
        out = g.partition() + g.input_arcs()
        g.close()
        return out

    serial = load(files, 1)
    for a, b in zip(serial, load(files, 8)):
        assert np.array_equal(a, b)
    # one ID record split over two lines: the chunked reader declines, the token reader agrees
    idf = open(files[1]).read().split("\n")
    idf[5] = idf[5].replace(" ", "\n", 1)
    split = str(tmp_path / "split_ID.txt")
    with open(split, "w") as f:
        f.write("\n".join(idf))
    for a, b in zip(serial, load((files[0], split, files[2]), 8)):
        assert np.array_equal(a, b)
    # a position given twice leaves another unset: not a permutation
    idf = open(files[1]).read().split("\n")
    first, second = idf[1].split(), idf[2].split()
    idf[2] = " ".join([first[0]] + second[1:])
    dup = str(tmp_path / "dup_ID.txt")
    with open(dup, "w") as f:
        f.write("\n".join(idf))
    for threads in (1, 8):
        rc, h = _load((files[0], dup, files[2]), H=8, Cg=2, threads=threads)
        assert rc == -3 and not h
