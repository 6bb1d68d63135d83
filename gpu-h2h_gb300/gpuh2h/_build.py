"""Compile the gpuh2h C-ABI library and the G2H command line for sm_103a.

Host translation units are compiled with g++, CUDA units with nvcc
(-gencode arch=compute_103a,code=sm_103a), all in parallel, then linked into
gpuh2h/_lib/libgpuh2h.so and gpuh2h/_lib/G2H.  Nothing is installed outside
the source tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                       # gpu-h2h_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libgpuh2h.so")
CLI = os.path.join(OUT, "G2H")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["io.cpp", "gen.cpp", "elim_sets.cu", "tree.cpp", "tree_gpu.cu", "capi.cpp", "contract.cu", "labels.cu", "query.cu", "noalloc.cu", "batch.cpp", "server.cpp", "loadgen.cpp", "index_io.cpp"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(nv))
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def build(force: bool = False, verbose: bool = False) -> str:
    """Build (incrementally) and return the path of libgpuh2h.so."""
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    hdrs = _headers()
    common_inc = ["-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(cuda, "include")]
    jobs = []
    objs = []
    for src in LIB_SOURCES + ["g2h_main.cpp"]:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJ, src + ".o")
        if src != "g2h_main.cpp":
            objs.append(obj)
        if not force and not _stale(obj, [path] + hdrs):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-ffp-contract=off",
                   *common_inc, "-c", path, "-o", obj]
        else:
            cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                   *common_inc, "-c", path, "-o", obj]
        jobs.append((cmd, obj))
    procs = []
    for cmd, obj in jobs:
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), cmd, obj))
    failed = []
    for p, cmd, obj in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("gpuh2h build failed:\n" + msg)
    libdir = os.path.join(cuda, "lib64")
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-L" + libdir, "-lcudart", "-lpthread"])
        os.replace(tmp, LIB)
    main_obj = os.path.join(OBJ, "g2h_main.cpp.o")
    if force or _stale(CLI, [LIB, main_obj]):
        tmp = CLI + ".tmp%d" % os.getpid()
        subprocess.check_call(["g++", "-o", tmp, main_obj, "-L" + OUT, "-lgpuh2h", "-L" + libdir, "-lcudart",
                               "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + libdir, "-lpthread"])
        os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
