"""Builds the CUDA library ``libaqua_gb300.so`` in-tree for sm_103a, then the
host runtime ``libaqua_host.so`` and the installable step tool
``libaqua_cuda_tool.so`` (``host/``, plain C++).

    python -m aquagpusph_gb300.build

Compiles the translation units of ``csrc/`` in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a``) and links them into
``aquagpusph_gb300/libaqua_gb300.so``.  ``-fmad=false`` keeps every multiply
and add a separate IEEE operation (no FMA contraction) and the default
``-prec-div=true -prec-sqrt=true`` keep divisions and square roots correctly
rounded: the arithmetic contract the reference's kernels are written in.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libaqua_gb300.so")
HOST = os.path.join(HERE, "host")
HOST_LIB = os.path.join(HERE, "libaqua_host.so")
TOOL_LIB = os.path.join(HERE, "libaqua_cuda_tool.so")
SOURCES = ("linklist.cu", "step.cu", "step_fast.cu", "api.cu", "noalloc.cu",
           "output.cu", "fastascii.cpp", "gnn.cu", "gnn_tc.cu")
# per-file arithmetic: the fast step kernels trade the reference's exact
# rounding for FMA contraction and approximate division / square root
FAST_MATH = {"step_fast.cu"}
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build "
                       "aquagpusph_gb300")


def _flags(src=""):
    math = ["-use_fast_math"] if src in FAST_MATH else ["-fmad=false"]
    return [ARCH, "-O3", "-lineinfo", "-std=c++17"] + math + [
        "-Xcompiler", "-fPIC", "-I", CSRC, "-I", os.path.join(ROOT, "include")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose=False, what="nvcc"):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(what + " failed:\n" + " ".join(cmd) + "\n" +
                           r.stdout + r.stderr)
    return r


def build_host(force: bool = False, verbose: bool = False) -> str:
    """The host runtime and the installable tool (needs libaqua_gb300.so)."""
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    inc = ["-I", HOST, "-I", os.path.join(ROOT, "include")]
    flags = ["-std=c++17", "-O2", "-fPIC", "-shared"]
    src = os.path.join(HOST, "aqua_host.cpp")
    hdrs = [os.path.join(HOST, "aqua_host.hpp"),
            os.path.join(ROOT, "include", "aqua_host.h")]
    if force or _stale(HOST_LIB, [src] + hdrs):
        _run([cxx] + flags + inc + [src, "-o", HOST_LIB, "-ldl"], verbose,
             "g++")
    tool = os.path.join(HOST, "aqua_cuda_tool.cpp")
    deps = [tool, HOST_LIB, LIB, os.path.join(ROOT, "include", "aqua_gb300.h")]
    if force or _stale(TOOL_LIB, deps + hdrs):
        _run([cxx] + flags + inc + [tool, "-o", TOOL_LIB, "-L", HERE,
                                    "-laqua_host", "-laqua_gb300",
                                    "-Wl,-rpath,$ORIGIN"], verbose, "g++")
    return TOOL_LIB


def build(force: bool = False, verbose: bool = False) -> str:
    objdir = os.path.join(ROOT, "_build", "aqua_gb300")
    os.makedirs(objdir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "aqua_gb300.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(objdir, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([cc] + _flags(src) + ["-c", s, "-o", o])

    def run(cmd):
        return _run(cmd, verbose)

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([cc, ARCH, "-shared", "-o", LIB] + objs)
    build_host(force, verbose)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
