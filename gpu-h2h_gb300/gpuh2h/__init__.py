"""gpuh2h -- Python mirror of the GPU-H2H operator interface over the C ABI.

The reference drives its hot path through Graph_D_H::Graph members called
from main.cu; `Graph` below keeps those names (contraction_noHub,
constructLabel_noHub, H2HDistancQuery_UsingLCA_noHub, ...) and their argument
meaning, and calls libgpuh2h.so (include/gpuh2h.h).  Device work needs the
CUDA build of the library; there is no CPU fallback: every compute call
raises if the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

H2H_OK = 0
LABEL_L3, LABEL_L4 = 3, 4
QUERY_LCA, QUERY_NOLCA = 0, 1
ERRORS = {-1: "ARG", -2: "IO", -3: "FORMAT", -4: "STATE", -5: "CUDA", -6: "NOMEM", -7: "UNSUPPORTED", -8: "DEVICE"}


class H2HError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class _Info(C.Structure):
    _fields_ = [(f, C.c_int32) for f in ("n", "partition_height", "change_height", "head", "tree_height",
                                          "n_levels", "gpu_vertices", "label_mode")] + \
               [(f, C.c_int64) for f in ("m", "label_size", "pos_size", "rmq_size", "euler_size", "lub_size",
                                          "adj_size", "device_bytes")] + \
               [(f, C.c_double) for f in ("lub_mb", "decomposition_tree_mb", "rmq_mb", "label_mb")] + \
               [(f, C.c_int64) for f in ("t_load_us", "t_rank_tree_us", "t_lub_us", "t_translate_lub_us",
                                          "t_td_gpu_us", "t_translate_back_us", "t_td_cpu_us", "t_tree_us",
                                          "t_malloc_us", "t_bfs_us", "t_translate_labels_us", "t_fill_gpu_us",
                                          "max_label", "label_updates")]


class _BatchInfo(C.Structure):
    _fields_ = [(f, C.c_int32) for f in ("graphs", "vertices", "elim_launches", "graph_captured")] + \
               [(f, C.c_int64) for f in ("fill_tiles", "device_bytes", "label_updates", "t_sets_us", "t_plan_us",
                                          "t_contract_us", "t_global_us", "t_download_us", "t_tree_us",
                                          "t_fill_plan_us", "t_fill_us", "t_attach_us", "t_total_us",
                                          "t_rebuild_us", "t_rebuild_fill_us")]


class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int32), ("poll_us", C.c_int32), ("slot_pairs", C.c_int64),
                ("memory_budget", C.c_int64)]


class _ServerStats(C.Structure):
    _fields_ = [(f, C.c_int64) for f in ("requests", "pairs", "batches", "max_inflight", "pending")] + \
               [("kernel_us", C.c_double), ("span_us", C.c_double), ("admitted_bytes", C.c_int64),
                ("memory_budget", C.c_int64)]


class LoadParams(C.Structure):
    _fields_ = [("rate", C.c_double), ("duration_s", C.c_double), ("size_lo", C.c_int64), ("size_hi", C.c_int64),
                ("requests", C.c_int64), ("inflight", C.c_int32), ("mode", C.c_int32), ("seed", C.c_uint64)]


class _LoadResult(C.Structure):
    _fields_ = [("requests", C.c_int64), ("pairs", C.c_int64), ("late", C.c_int64), ("wall_s", C.c_double)]


class GenParams(C.Structure):
    _fields_ = [("n", C.c_int64), ("cols", C.c_int32), ("aspect_milli", C.c_int32), ("jitter_milli", C.c_int32),
                ("drop_permille", C.c_int32), ("target_arcs", C.c_int64), ("diag_permille", C.c_int32),
                ("hw_tiers", C.c_int32), ("hw_permille10", C.c_int32), ("hw_k", C.c_int32),
                ("hw_scale_milli", C.c_int32), ("weight_max", C.c_int32), ("partition_height", C.c_int32),
                ("seed", C.c_uint64)]


# Exported symbols and their ctypes signatures (kept in step with include/*.h).
_vp, _i32, _i64, _cp = C.c_void_p, C.c_int, C.c_int64, C.c_char_p
SIGNATURES = {
    "h2h_load": (_i32, [_cp, _cp, _i32, _i32, _i32, _i32, C.POINTER(_vp)]),
    "h2h_load_files": (_i32, [_cp, _cp, _cp, _cp, _i32, _i32, _i32, _i32, C.POINTER(_vp)]),
    "h2h_free": (None, [_vp]),
    "h2h_last_error": (_cp, []),
    "h2h_contract": (_i32, [_vp, _i32]),
    "h2h_build_labels": (_i32, [_vp, _i32, _i32, _i32]),
    "h2h_query_lca_nohub": (_i32, [_vp, _i32, _i32]),
    "h2h_query_nolca_nohub": (_i32, [_vp, _i32, _i32]),
    "h2h_query_batch": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp]),
    "h2h_query_batch_host": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32]),
    "h2h_query_batch_plain": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp]),
    "h2h_get_info": (_i32, [_vp, C.POINTER(_Info)]),
    "h2h_copy_order": (_i32, [_vp, _vp]),
    "h2h_copy_tree": (_i32, [_vp, _vp, _vp, _vp]),
    "h2h_copy_rmq": (_i32, [_vp, _vp, _vp]),
    "h2h_copy_adj": (_i32, [_vp, _vp, _vp, _vp]),
    "h2h_copy_labels": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "h2h_copy_bfs": (_i32, [_vp, _vp, _vp]),
    "h2h_write_partition_rate": (_i32, [_vp, _cp]),
    "h2h_write_contract_csv": (_i32, [_vp, _cp]),
    "h2h_write_construct_info": (_i32, [_vp, _cp]),
    "h2h_write_query_result": (_i32, [_vp, _cp, _i64, _vp]),
    "h2h_gen_default": (None, [C.POINTER(GenParams)]),
    "h2h_generate_road": (_i32, [C.POINTER(GenParams), _cp, _cp, C.POINTER(_i64)]),
    "h2h_gen_uniform_pairs": (_i32, [_i32, _i64, C.c_uint64, _vp, _vp]),
    "h2h_gen_local_pairs": (_i32, [_vp, _i64, _i32, C.c_uint64, _vp, _vp]),
    "h2h_fill_labels_l4_noalloc": (_i32, [_i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _i32, _i32,
                                          _vp]),
    "h2h_copy_input_arcs": (_i32, [_vp, _vp, _vp, _vp]),
    "h2h_copy_partition": (_i32, [_vp, _vp, _vp]),
    "h2h_save_index": (_i32, [_vp, _cp]),
    "h2h_fill_labels_plain": (_i32, [_vp, C.POINTER(C.c_double), C.POINTER(_i64)]),
    "h2h_fill_labels_plain_node": (_i32, [_vp, C.POINTER(C.c_double), C.POINTER(_i64)]),
    "h2h_load_index": (_i32, [_cp, C.POINTER(_vp)]),
    "h2h_batch_build": (_i32, [_vp, _i32, _i32, C.POINTER(_vp)]),
    "h2h_batch_set_weights": (_i32, [_vp, _i32, _vp]),
    "h2h_batch_rebuild": (_i32, [_vp]),
    "h2h_batch_sync_host": (_i32, [_vp]),
    "h2h_batch_set_policy": (_i32, [_vp, _cp]),
    "h2h_batch_get_policy": (_i32, [_vp, _vp, _i32]),
    "h2h_batch_tune": (_i32, [_vp, _i32, _vp, _i32]),
    "h2h_batch_get_info": (_i32, [_vp, C.POINTER(_BatchInfo)]),
    "h2h_batch_free": (None, [_vp]),
    "h2h_server_default_config": (None, [C.POINTER(ServerConfig)]),
    "h2h_server_create": (_i32, [C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "h2h_server_add_graph": (_i32, [_vp, _vp, C.POINTER(_i32)]),
    "h2h_server_remove_graph": (_i32, [_vp, _i32]),
    "h2h_server_submit": (_i32, [_vp, _i32, _vp, _vp, _vp, _i64, _i32, C.POINTER(C.c_uint64)]),
    "h2h_server_wait": (_i32, [_vp, C.c_uint64, _i64]),
    "h2h_server_test": (_i32, [_vp, C.c_uint64]),
    "h2h_server_release": (_i32, [_vp, C.c_uint64, C.POINTER(C.c_double)]),
    "h2h_server_get_stats": (_i32, [_vp, C.POINTER(_ServerStats)]),
    "h2h_server_reset_stats": (_i32, [_vp]),
    "h2h_server_free": (None, [_vp]),
    "h2h_server_load": (_i32, [_vp, _vp, _vp, _i32, C.POINTER(LoadParams), _vp, _vp, _vp, _i64,
                               C.POINTER(_LoadResult)]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load_library(build: bool = True):
    """Load libgpuh2h.so (building it first when `build`)."""
    global _lib
    if _lib is None:
        path = _build.build() if build else _build.LIB
        if not os.path.exists(path):
            raise OSError("libgpuh2h.so is not built (%s)" % path)
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int):
    if rc != H2H_OK:
        raise H2HError(rc, load_library().h2h_last_error().decode())


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _require_gpu():
    try:
        import torch
        ok = torch.cuda.is_available()
    except Exception:  # torch is plumbing only; the library itself does not need it
        ok = True
    if not ok:
        raise H2HError(-5, "no CUDA device: the GPU hot path has no CPU fallback")


PARTITION_PREFIX = {1: "Latitude", 2: "Minimum", 3: "metis", 4: "scotch"}


class Graph:
    """One road graph through the hot path, mirroring Graph_D_H::Graph.

    Graph(graphName, TreeHeight, changeHeight, threadNum, partitionMethod,
    root=".") loads <root>/Graph/USA/<G>Edge.txt and the partition files the
    same way main.cu:262-296 builds the paths.
    """

    def __init__(self, graphName: str, TreeHeight: int, changeHeight: int, threadNum: int = 8,
                 partitionMethod: int = 1, root: str = ".", files: tuple | None = None):
        L = load_library()
        self._L = L
        h = C.c_void_p()
        if files is not None:
            edge, idf, cut = files
            rc = L.h2h_load_files(edge.encode(), idf.encode(), cut.encode(), graphName.encode(), TreeHeight,
                                  changeHeight, threadNum, partitionMethod, C.byref(h))
        else:
            rc = L.h2h_load(root.encode(), graphName.encode(), TreeHeight, changeHeight, threadNum,
                            partitionMethod, C.byref(h))
        _check(rc)
        self.h = h
        self.graphName = graphName

    @classmethod
    def load_index(cls, path: str, graphName: str = "index") -> "Graph":
        """A built index read back from h2h_save_index's file (no rebuild)."""
        L = load_library()
        h = C.c_void_p()
        _check(L.h2h_load_index(path.encode(), C.byref(h)))
        g = cls.__new__(cls)
        g._L = L
        g.h = h
        g.graphName = graphName
        return g

    def fill_labels_plain(self, mapping: str = "pair"):
        """(device ms, mismatching entries) of one of the reference's GPU fill
        mappings re-run on this graph (measurement baseline): "pair", a
        thread per (v, u) pair (parallelFine = 2), or "node", a thread per
        node (parallelFine = 1)."""
        ms = C.c_double()
        bad = C.c_int64()
        fn = {"pair": self._L.h2h_fill_labels_plain, "node": self._L.h2h_fill_labels_plain_node}[mapping]
        _check(fn(self.h, C.byref(ms), C.byref(bad)))
        return ms.value, bad.value

    def save_index(self, path: str):
        _check(self._L.h2h_save_index(self.h, path.encode()))

    def close(self):
        if getattr(self, "h", None):
            self._L.h2h_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # main.cu:149-158
    def contraction_noHub(self, contractDevice: int = 1):
        _require_gpu()
        _check(self._L.h2h_contract(self.h, contractDevice))
        return self

    # main.cu:160-188
    def constructLabel_noHub(self, parallelFine: int = 2, constructDevice: int = 1, label_mode: int = LABEL_L4):
        _require_gpu()
        _check(self._L.h2h_build_labels(self.h, parallelFine, constructDevice, label_mode))
        return self

    # Query.cu:108 / :124
    def H2HDistancQuery_UsingLCA_noHub(self, x: int, y: int) -> int:
        r = self._L.h2h_query_lca_nohub(self.h, int(x), int(y))
        if r < 0:
            raise H2HError(-1, self._L.h2h_last_error().decode())
        return r

    def H2HDistancQuery_noLCA_noHub(self, x: int, y: int) -> int:
        r = self._L.h2h_query_nolca_nohub(self.h, int(x), int(y))
        if r < 0:
            raise H2HError(-1, self._L.h2h_last_error().decode())
        return r

    # kernel_functions.cuh:94-127 over host arrays (copies in, kernel, copies out)
    def query(self, x, y, mode: int = QUERY_LCA) -> np.ndarray:
        x = np.ascontiguousarray(x, np.int32)
        y = np.ascontiguousarray(y, np.int32)
        out = np.empty(len(x), np.int32)
        _check(self._L.h2h_query_batch_host(self.h, _p(x), _p(y), _p(out), len(x), mode))
        return out

    def H2HQuery_UsingLCA_noHub(self, x_ptr: int, y_ptr: int, out_ptr: int, n: int, stream: int = 0):
        """Device-pointer batch on a caller stream (torch tensors: .data_ptr(), stream.cuda_stream)."""
        _check(self._L.h2h_query_batch(self.h, x_ptr, y_ptr, out_ptr, n, QUERY_LCA, stream or None))

    def H2HQuery_noLCA_noHub(self, x_ptr: int, y_ptr: int, out_ptr: int, n: int, stream: int = 0):
        _check(self._L.h2h_query_batch(self.h, x_ptr, y_ptr, out_ptr, n, QUERY_NOLCA, stream or None))

    def query_device(self, x_ptr: int, y_ptr: int, out_ptr: int, n: int, mode: int = QUERY_LCA, stream: int = 0):
        _check(self._L.h2h_query_batch(self.h, x_ptr, y_ptr, out_ptr, n, mode, stream or None))

    def query_device_plain(self, x_ptr: int, y_ptr: int, out_ptr: int, n: int, mode: int = QUERY_LCA,
                           stream: int = 0):
        """The reference's one-thread-per-query mapping (measurement baseline)."""
        _check(self._L.h2h_query_batch_plain(self.h, x_ptr, y_ptr, out_ptr, n, mode, stream or None))

    def query_host_ptr(self, x_ptr: int, y_ptr: int, out_ptr: int, n: int, mode: int = QUERY_LCA):
        """h2h_query_batch_host on raw host pointers (e.g. pinned torch tensors)."""
        _check(self._L.h2h_query_batch_host(self.h, x_ptr, y_ptr, out_ptr, n, mode))

    # ---- accessors for parity tests
    def info(self) -> dict:
        inf = _Info()
        _check(self._L.h2h_get_info(self.h, C.byref(inf)))
        return {f: getattr(inf, f) for f, _ in _Info._fields_}

    def order(self) -> np.ndarray:
        a = np.empty(self.info()["n"], np.int32)
        _check(self._L.h2h_copy_order(self.h, _p(a)))
        return a

    def tree(self):
        n = self.info()["n"]
        f, d, fi = (np.empty(n, np.int32) for _ in range(3))
        _check(self._L.h2h_copy_tree(self.h, _p(f), _p(d), _p(fi)))
        return f, d, fi

    def rmq(self):
        i = self.info()
        h = np.empty(i["euler_size"], np.int64)
        r = np.empty(i["rmq_size"], np.int32)
        _check(self._L.h2h_copy_rmq(self.h, _p(h), _p(r)))
        return h, r

    def adj(self):
        i = self.info()
        ah = np.empty(i["n"] + 1, np.int64)
        aid = np.empty(i["adj_size"], np.int32)
        aw = np.empty(i["adj_size"], np.int32)
        _check(self._L.h2h_copy_adj(self.h, _p(ah), _p(aid), _p(aw)))
        return ah, aid, aw

    def labels(self) -> dict:
        i = self.info()
        n = i["n"]
        dh = np.empty(n + 1, np.int64)
        dis = np.empty(i["label_size"], np.int32)
        ph = np.empty(n + 1, np.int64)
        pid = np.empty(i["pos_size"], np.int32)
        pp = np.empty(i["pos_size"], np.int32)
        _check(self._L.h2h_copy_labels(self.h, _p(dh), _p(dis), _p(ph), _p(pid), _p(pp)))
        return dict(dis_hash=dh, dis=dis, pos_hash=ph, pos_id=pid, pos_pos=pp)

    def labels_pos_hash(self) -> np.ndarray:
        """H2H_pos_hash only (no label download)."""
        ph = np.empty(self.info()["n"] + 1, np.int64)
        _check(self._L.h2h_copy_labels(self.h, None, None, _p(ph), None, None))
        return ph

    def bfs(self):
        i = self.info()
        tb = np.empty(i["n"], np.int32)
        th = np.empty(i["n_levels"] + 1, np.int32)
        _check(self._L.h2h_copy_bfs(self.h, _p(tb), _p(th)))
        return tb, th

    def input_arcs(self):
        """Stored arcs in CSR order (the order h2h_batch_set_weights takes)."""
        i = self.info()
        off = np.empty(i["n"] + 1, np.int32)
        v = np.empty(i["m"], np.int32)
        w = np.empty(i["m"], np.int32)
        _check(self._L.h2h_copy_input_arcs(self.h, _p(off), _p(v), _p(w)))
        return off, v, w

    def partition(self):
        """(part_ids, id_hash): the vertex at each partition position and the
        position of each vertex, as the ID file gives them."""
        n = self.info()["n"]
        part = np.empty(n, np.int32)
        pos = np.empty(n, np.int32)
        _check(self._L.h2h_copy_partition(self.h, _p(part), _p(pos)))
        return part, pos

    def local_pairs(self, n: int, max_hops: int = 20, seed: int = 1):
        x = np.empty(n, np.int32)
        y = np.empty(n, np.int32)
        _check(self._L.h2h_gen_local_pairs(self.h, n, max_hops, seed, _p(x), _p(y)))
        return x, y

    # ---- CSV outputs with the reference's schemas
    def write_partition_rate(self, directory: str = "."):
        _check(self._L.h2h_write_partition_rate(self.h, directory.encode()))

    def write_contract_csv(self, root: str = "."):
        _check(self._L.h2h_write_contract_csv(self.h, root.encode()))

    def printConstructInfo(self, root: str = "."):
        _check(self._L.h2h_write_construct_info(self.h, root.encode()))

    def write_query_result(self, root: str, query_number: int, times_us):
        t = np.zeros(18, np.int64)
        t[:len(times_us)] = times_us
        _check(self._L.h2h_write_query_result(self.h, root.encode(), query_number, _p(t)))


class Batch:
    """Several loaded graphs contracted and labelled together (h2h_batch_*).

    Batch(graphs, threads) builds every graph; afterwards each Graph answers
    queries on its own.  The Graph objects must stay open while the batch
    lives (the batch keeps references to them).
    """

    def __init__(self, graphs, threads: int = 8):
        _require_gpu()
        L = load_library()
        self._L = L
        self.graphs = list(graphs)
        arr = (C.c_void_p * len(self.graphs))(*[g.h for g in self.graphs])
        b = C.c_void_p()
        _check(L.h2h_batch_build(C.cast(arr, C.c_void_p), len(self.graphs), threads, C.byref(b)))
        self.b = b

    def close(self):
        if getattr(self, "b", None):
            self._L.h2h_batch_free(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        inf = _BatchInfo()
        _check(self._L.h2h_batch_get_info(self.b, C.byref(inf)))
        return {f: getattr(inf, f) for f, _ in _BatchInfo._fields_}

    def set_weights(self, index: int, w: np.ndarray):
        w = np.ascontiguousarray(w, np.int32)
        _check(self._L.h2h_batch_set_weights(self.b, index, _p(w)))

    def rebuild(self):
        _check(self._L.h2h_batch_rebuild(self.b))

    def sync_host(self):
        _check(self._L.h2h_batch_sync_host(self.b))

    def policy(self) -> str:
        buf = C.create_string_buffer(512)
        _check(self._L.h2h_batch_get_policy(self.b, C.cast(buf, C.c_void_p), 512))
        return buf.value.decode()

    def set_policy(self, policy: str):
        _check(self._L.h2h_batch_set_policy(self.b, policy.encode()))

    def tune(self, rounds: int = 1) -> str:
        buf = C.create_string_buffer(512)
        _check(self._L.h2h_batch_tune(self.b, rounds, C.cast(buf, C.c_void_p), 512))
        return buf.value.decode()


class Server:
    """Continuous-batching query server over resident graphs (h2h_server_*).

    Server(slots=4, slot_pairs=1 << 20); add(graph) -> id; submit(id, x, y,
    out) -> request (x, y, out: int32 numpy arrays kept alive until release);
    wait(request); release(request) -> latency in us.
    """

    def __init__(self, slots: int = 4, slot_pairs: int = 1 << 20, poll_us: int = 5, memory_budget: int = 0):
        _require_gpu()
        L = load_library()
        self._L = L
        c = ServerConfig()
        L.h2h_server_default_config(C.byref(c))
        c.slots, c.slot_pairs, c.poll_us, c.memory_budget = slots, slot_pairs, poll_us, memory_budget
        s = C.c_void_p()
        _check(L.h2h_server_create(C.byref(c), C.byref(s)))
        self.s = s
        self._graphs = []
        self._live = {}

    def close(self):
        if getattr(self, "s", None):
            self._L.h2h_server_free(self.s)
            self.s = None
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, graph: "Graph") -> int:
        gid = C.c_int()
        _check(self._L.h2h_server_add_graph(self.s, graph.h, C.byref(gid)))
        self._graphs.append(graph)
        return gid.value

    def remove(self, gid: int):
        _check(self._L.h2h_server_remove_graph(self.s, gid))

    def submit(self, gid: int, x: np.ndarray, y: np.ndarray, out: np.ndarray, mode: int = QUERY_LCA) -> int:
        for a in (x, y, out):
            assert a.dtype == np.int32 and a.flags.c_contiguous
        rid = C.c_uint64()
        _check(self._L.h2h_server_submit(self.s, gid, _p(x), _p(y), _p(out), len(x), mode, C.byref(rid)))
        self._live[rid.value] = (x, y, out)
        return rid.value

    def wait(self, rid: int, timeout_us: int = -1):
        _check(self._L.h2h_server_wait(self.s, rid, timeout_us))

    def done(self, rid: int) -> bool:
        r = self._L.h2h_server_test(self.s, rid)
        if r < 0:
            _check(r)
        return r == 1

    def release(self, rid: int) -> float:
        lat = C.c_double()
        _check(self._L.h2h_server_release(self.s, rid, C.byref(lat)))
        self._live.pop(rid, None)
        return lat.value

    def stats(self) -> dict:
        st = _ServerStats()
        _check(self._L.h2h_server_get_stats(self.s, C.byref(st)))
        return {f: getattr(st, f) for f, _ in _ServerStats._fields_}

    def reset_stats(self):
        _check(self._L.h2h_server_reset_stats(self.s))

    def load(self, gids, n_vertices, rate: float = 0.0, duration_s: float = 1.0, size_lo: int = 1,
             size_hi: int = 100_000, requests: int = 0, inflight: int = 1, mode: int = QUERY_LCA, seed: int = 1,
             max_requests: int = 1_000_000) -> dict:
        """Drive the server with h2h_server_load; returns per-request latency
        (us, from scheduled arrival), sizes and graph indices."""
        g = np.ascontiguousarray(gids, np.int32)
        nv = np.ascontiguousarray(n_vertices, np.int32)
        p = LoadParams(rate, duration_s, size_lo, size_hi, requests, inflight, mode, seed)
        lat = np.zeros(max_requests, np.float64)
        sz = np.zeros(max_requests, np.int64)
        go = np.zeros(max_requests, np.int32)
        r = _LoadResult()
        _check(self._L.h2h_server_load(self.s, _p(g), _p(nv), len(g), C.byref(p), _p(lat), _p(sz), _p(go),
                                       max_requests, C.byref(r)))
        k = min(r.requests, max_requests)
        return dict(requests=r.requests, pairs=r.pairs, late=r.late, wall_s=r.wall_s, latency_us=lat[:k],
                    sizes=sz[:k], graph=go[:k])


def gen_params(**kw) -> GenParams:
    p = GenParams()
    load_library().h2h_gen_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def generate_road(root: str, name: str, **kw) -> int:
    """Write a seeded synthetic road graph in the reference formats; returns the arc count."""
    p = gen_params(**kw)
    arcs = C.c_int64()
    _check(load_library().h2h_generate_road(C.byref(p), root.encode(), name.encode(), C.byref(arcs)))
    return arcs.value


def road_batch_params(count: int = 64, n_lo: int = 2000, n_hi: int = 200000, seed: int = 7) -> list:
    """Generator parameters of `count` road graphs with vertex counts drawn
    log-uniform in [n_lo, n_hi] (seeded), the 264,346-vertex road graph's
    shape (jittered 1:1.3 grid, 2.776 arcs per vertex, 0.5% highway layer),
    partition height ceil(log2(n / 256)) (at least 2)."""
    import math
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        out.append(dict(n=n, target_arcs=int(round(n * 733846 / 264346)), aspect_milli=1300, jitter_milli=300,
                        diag_permille=50, hw_tiers=1, hw_permille10=50, hw_k=3, hw_scale_milli=400,
                        partition_height=max(2, math.ceil(math.log2(n / 256))), seed=1000 + i, cols=0,
                        drop_permille=0))
    return out


def write_edge_file(path: str, off: np.ndarray, v: np.ndarray, w: np.ndarray):
    """An Edge file (1-based `a u v w` lines) holding the stored arcs in CSR
    order, so a graph loaded from it has exactly these arcs."""
    n = len(off) - 1
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(off.astype(np.int64)))
    with open(path, "w") as f:
        f.write("%d %d\n" % (n, len(v)))
        f.write("".join("a %d %d %d\n" % (a + 1, b + 1, c) for a, b, c in zip(src, v, w)))


def uniform_pairs(n_vertices: int, n: int, seed: int = 1):
    x = np.empty(n, np.int32)
    y = np.empty(n, np.int32)
    _check(load_library().h2h_gen_uniform_pairs(n_vertices, n, seed, _p(x), _p(y)))
    return x, y


def files_for(root: str, name: str, method: int = 1):
    pre = os.path.join(root, "Partition", name, PARTITION_PREFIX[method])
    return (os.path.join(root, "Graph", "USA", name + "Edge.txt"), pre + "ID.txt", pre + "Cut.txt")


def fill_labels_l4_noalloc(n: int, order: int, father: int, depth: int, pos_hash: int, pos_id: int, pos_pos: int,
                           pos_w: int, dis_hash: int, total_label: int, dis: int, max_depth: int, max_sep: int,
                           stream: int = 0):
    """h2h_fill_labels_l4_noalloc on device pointers: the L4 label fill for
    callers that cannot allocate device memory (scratch in a fixed on-device
    array; see include/gpuh2h.h for the size limit)."""
    _check(load_library().h2h_fill_labels_l4_noalloc(n, order, father, depth, pos_hash, pos_id, pos_pos, pos_w,
                                                      dis_hash, total_label, dis, max_depth, max_sep,
                                                      stream or None))
