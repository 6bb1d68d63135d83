"""ctypes binding of the C oracle (h2h_oracle.c) and the reference harness.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / reference arm, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


PKG_CSRC = os.path.join(os.path.dirname(HERE), "gpu-h2h_gb300", "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")


def build(force: bool = False) -> str:
    """Compile oracle/_build/liboracle.so: h2h_oracle.c (gcc, plain C) plus
    the workload generators (the library's gen.cpp and gen_shim.cpp, g++),
    so a CPU-only run needs nothing from the GPU library."""
    srcs = [os.path.join(HERE, "h2h_oracle.c"), os.path.join(HERE, "gen_shim.cpp"),
            os.path.join(PKG_CSRC, "gen.cpp")]
    deps = srcs + [os.path.join(HERE, "h2h_oracle.h"), os.path.join(PKG_CSRC, "gen.h"),
                   os.path.join(PKG_CSRC, "status.h"), os.path.join(INCLUDE, "gpuh2h_tools.h"),
                   os.path.join(INCLUDE, "gpuh2h.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I" + HERE, "-I" + PKG_CSRC, "-I" + INCLUDE]
    tag = "%d" % os.getpid()
    objs = [os.path.join(BUILD, os.path.basename(x) + "." + tag + ".o") for x in srcs]
    procs = [subprocess.Popen(["gcc", "-std=c11", "-O2", "-fPIC", "-c", srcs[0], "-o", objs[0]])]
    for src, obj in zip(srcs[1:], objs[1:]):
        procs.append(subprocess.Popen(["g++", "-std=c++17", "-O2", "-fPIC", *inc, "-c", src, "-o", obj]))
    if any(p.wait() != 0 for p in procs):
        raise RuntimeError("oracle build failed")
    tmp = LIB + ".tmp" + tag
    subprocess.check_call(["g++", "-shared", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


class GenParams(C.Structure):
    """h2h_gen_params (include/gpuh2h_tools.h)."""
    _fields_ = [("n", C.c_int64), ("cols", C.c_int32), ("aspect_milli", C.c_int32), ("jitter_milli", C.c_int32),
                ("drop_permille", C.c_int32), ("target_arcs", C.c_int64), ("diag_permille", C.c_int32),
                ("hw_tiers", C.c_int32), ("hw_permille10", C.c_int32), ("hw_k", C.c_int32),
                ("hw_scale_milli", C.c_int32), ("weight_max", C.c_int32), ("partition_height", C.c_int32),
                ("seed", C.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
        L.or_load.restype = vp
        L.or_load.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, i32, i32, i32]
        L.or_free.argtypes = [vp]
        L.or_error.restype = C.c_char_p
        L.or_error.argtypes = [vp]
        L.or_contract.argtypes = [vp]
        L.or_build_labels.argtypes = [vp, i32, i32]
        L.or_query_lca.argtypes = [vp, i32, i32]
        L.or_query_nolca.argtypes = [vp, i32, i32]
        L.or_query_batch.argtypes = [vp, vp, vp, vp, i64, i32, i32]
        L.or_dijkstra.argtypes = [vp, i32, vp]
        for name in ("or_n", "or_tree_height", "or_n_levels", "or_head", "or_gpu_vertices"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = i32
        for name in ("or_label_size", "or_pos_size", "or_rmq_size", "or_euler_size", "or_lub_size",
                     "or_adj_total"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = i64
        for name in ("or_get_order", "or_get_father", "or_get_depth", "or_get_first"):
            getattr(L, name).argtypes = [vp, vp]
        L.or_get_rmq.argtypes = [vp, vp, vp]
        L.or_get_labels.argtypes = [vp, vp, vp, vp, vp, vp]
        L.or_get_bfs.argtypes = [vp, vp, vp]
        L.or_get_adj.argtypes = [vp, vp, vp, vp]
        L.or_input_arcs.argtypes = [vp]
        L.or_input_arcs.restype = i64
        L.or_get_input_arcs.argtypes = [vp, vp, vp]
        L.or_gen_default.argtypes = [vp]
        L.or_generate_road.argtypes = [vp, C.c_char_p, C.c_char_p, C.POINTER(i64), C.c_char_p, i32]
        L.or_gen_uniform_pairs.argtypes = [i32, i64, C.c_uint64, vp, vp]
        L.or_gen_local_pairs.argtypes = [vp, i64, i32, C.c_uint64, vp, vp]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class OracleGraph:
    """The reference pipeline restated on the CPU: load, GPU-hybrid
    contraction (restated kernel + global heap), tree/RMQ, labels, queries."""

    def __init__(self, edge: str, idf: str, cut: str, H: int, Cg: int, threads: int = 4):
        L = lib()
        self._L = L
        self.h = L.or_load(edge.encode(), idf.encode(), cut.encode(), H, Cg, threads)
        if not self.h:
            raise IOError("oracle could not load %s / %s / %s" % (edge, idf, cut))
        self.threads = threads

    def close(self):
        if self.h:
            self._L.or_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def contract(self):
        if self._L.or_contract(self.h) != 0:
            raise RuntimeError(self._L.or_error(self.h).decode())
        return self

    def build_labels(self, l4: bool = True, threads: int | None = None):
        if self._L.or_build_labels(self.h, 1 if l4 else 0, threads or self.threads) != 0:
            raise RuntimeError(self._L.or_error(self.h).decode())
        return self

    @property
    def n(self) -> int:
        return self._L.or_n(self.h)

    def _arr(self, fn, n, dt):
        a = np.empty(n, dtype=dt)
        fn(self.h, _p(a))
        return a

    def order(self):
        return self._arr(self._L.or_get_order, self.n, np.int32)

    def father(self):
        return self._arr(self._L.or_get_father, self.n, np.int32)

    def depth(self):
        return self._arr(self._L.or_get_depth, self.n, np.int32)

    def first(self):
        return self._arr(self._L.or_get_first, self.n, np.int32)

    def rmq(self):
        L = self._L
        h = np.empty(L.or_euler_size(self.h), dtype=np.int64)
        i = np.empty(L.or_rmq_size(self.h), dtype=np.int32)
        L.or_get_rmq(self.h, _p(h), _p(i))
        return h, i

    def labels(self):
        L, n = self._L, self.n
        dh = np.empty(n + 1, np.int64)
        dis = np.empty(L.or_label_size(self.h), np.int32)
        ph = np.empty(n + 1, np.int64)
        pid = np.empty(L.or_pos_size(self.h), np.int32)
        pp = np.empty(L.or_pos_size(self.h), np.int32)
        L.or_get_labels(self.h, _p(dh), _p(dis), _p(ph), _p(pid), _p(pp))
        return dict(dis_hash=dh, dis=dis, pos_hash=ph, pos_id=pid, pos_pos=pp)

    def bfs(self):
        L, n = self._L, self.n
        tb = np.empty(n, np.int32)
        th = np.empty(L.or_n_levels(self.h) + 1, np.int32)
        L.or_get_bfs(self.h, _p(tb), _p(th))
        return tb, th

    def adj(self):
        L, n = self._L, self.n
        t = L.or_adj_total(self.h)
        ah = np.empty(n + 1, np.int64)
        aid = np.empty(t, np.int32)
        aw = np.empty(t, np.int32)
        L.or_get_adj(self.h, _p(ah), _p(aid), _p(aw))
        return ah, aid, aw

    def query(self, x: int, y: int, lca: bool = True) -> int:
        return (self._L.or_query_lca if lca else self._L.or_query_nolca)(self.h, int(x), int(y))

    def query_batch(self, x, y, lca: bool = True, threads: int | None = None):
        x = np.ascontiguousarray(x, np.int32)
        y = np.ascontiguousarray(y, np.int32)
        out = np.empty(len(x), np.int32)
        self._L.or_query_batch(self.h, _p(x), _p(y), _p(out), len(x), 0 if lca else 1,
                               threads or self.threads)
        return out

    def local_pairs(self, n: int, max_hops: int = 20, seed: int = 1):
        """The library's local-pair generator over this graph's input arcs."""
        x = np.empty(n, np.int32)
        y = np.empty(n, np.int32)
        if self._L.or_gen_local_pairs(self.h, n, max_hops, seed, _p(x), _p(y)) != 0:
            raise ValueError("bad local-pair arguments")
        return x, y

    def input_arcs(self):
        n = self.n
        off = np.empty(n + 1, np.int32)
        v = np.empty(self._L.or_input_arcs(self.h), np.int32)
        self._L.or_get_input_arcs(self.h, _p(off), _p(v))
        return off, v

    def dijkstra(self, src: int):
        d = np.empty(self.n, np.int32)
        self._L.or_dijkstra(self.h, int(src), _p(d))
        return d

    def summary(self) -> dict:
        L = self._L
        return dict(n=self.n, head=L.or_head(self.h), tree_height=L.or_tree_height(self.h),
                    label_size=L.or_label_size(self.h), pos_size=L.or_pos_size(self.h),
                    rmq_size=L.or_rmq_size(self.h), lub=L.or_lub_size(self.h),
                    gpu_vertices=L.or_gpu_vertices(self.h), levels=L.or_n_levels(self.h))


def generate_road(root: str, name: str, **kw) -> int:
    """The library's seeded road-graph generator (same bytes as
    gpuh2h.generate_road); returns the arc count."""
    L = lib()
    p = GenParams()
    L.or_gen_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    arcs = C.c_int64()
    msg = C.create_string_buffer(512)
    rc = L.or_generate_road(C.byref(p), root.encode(), name.encode(), C.byref(arcs), msg, 512)
    if rc != 0:
        raise RuntimeError("generator: %s" % msg.value.decode())
    return arcs.value


def uniform_pairs(n_vertices: int, n: int, seed: int = 1):
    x = np.empty(n, np.int32)
    y = np.empty(n, np.int32)
    if lib().or_gen_uniform_pairs(n_vertices, n, seed, _p(x), _p(y)) != 0:
        raise ValueError("bad pair arguments")
    return x, y


def build_ref_gpu() -> bool:
    """Build the reference's own GPU code (oracle/build_ref_gpu.sh --build)
    from the staged sources; False where nothing was staged."""
    rc = subprocess.call([os.path.join(HERE, "build_ref_gpu.sh"), "--build"], stdout=subprocess.DEVNULL)
    if rc == 3:
        return False
    if rc != 0:
        raise RuntimeError("build_ref_gpu.sh --build failed (exit %d)" % rc)
    return True


def run_reference(edge, idf, cut, H, Cg, threads=4, l4=True, pairs=None, gpu=False):
    """Run a build of the reference and return its dumped arrays.

    gpu=False: the CPU build (oracle/_ref/ref_harness_L{3,4}, build_ref.sh).
    gpu=True: the reference's own GPU kernels built for sm_103a
    (oracle/_ref/ref_gpu_harness_L4, build_ref_gpu.sh): GPU partition
    contraction, GPU LL label fill with the L4 walk, GPU batched queries;
    its phase timers come back under "times" (microseconds)."""
    if gpu:
        if not l4:
            raise ValueError("the GPU harness is built with the L4 label kernel only")
        exe = os.path.join(REF_DIR, "ref_gpu_harness_L4")
    else:
        exe = os.path.join(REF_DIR, "ref_harness_L4" if l4 else "ref_harness_L3")
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    with tempfile.TemporaryDirectory() as wd:
        out = os.path.join(wd, "out")
        os.makedirs(out)
        args = [exe, os.path.abspath(edge), os.path.abspath(idf), os.path.abspath(cut), str(H), str(Cg),
                str(threads), out]
        if pairs is not None:
            pf = os.path.join(wd, "pairs.i32")
            np.ascontiguousarray(pairs, np.int32).tofile(pf)
            args.append(pf)
        subprocess.run(args, cwd=wd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
                       timeout=600)
        res = {}
        for f in os.listdir(out):
            name, ext = f.rsplit(".", 1)
            if ext == "txt":
                res[name] = {k: int(v) for k, v in (line.split() for line in open(os.path.join(out, f)) if line.strip())}
            else:
                res[name] = np.fromfile(os.path.join(out, f), dtype=np.int32 if ext == "i32" else np.int64)
        return res
