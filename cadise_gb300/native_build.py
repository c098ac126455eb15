"""In-tree build of the CUDA library ``cadise_gb300/_build/libcadise_gpu.so``.

Every translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked with
the static CUDA runtime.  No CMake.  Used by ``__graft_entry__.build()`` and
the test suite; rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.abspath(os.path.join(HERE, "..", "include"))
LIB = os.path.join(BUILD, "libcadise_gpu.so")
CLI = os.path.join(BUILD, "cadise-gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# No contraction of a * b + c into one fused multiply-add: every kernel then
# rounds each product and sum the way the reference's FP32 code does, and the
# same inlined function rounds identically in every kernel it lands in (the
# wavefront and the megakernel agree path for path).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-pthread"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(_nvcc()))), "include")


def sources():
    out = []
    for d in (CSRC, HOST):
        out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cu", ".cpp")) and f != "cli.cpp"]
    return sorted(out)


def headers():
    hs = []
    for d in (CSRC, HOST, INCLUDE):
        hs += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cuh", ".h"))]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + headers()):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + ["-I", INCLUDE, "-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-I", INCLUDE, "-I", _cuda_include(), "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False, jobs: int = 0) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [_nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    cli_src = os.path.join(HOST, "cli.cpp")
    if _stale(CLI, [cli_src, LIB] + headers()):
        cmd = ["g++"] + CXX_FLAGS + ["-I", INCLUDE, "-I", _cuda_include(), cli_src, "-o", CLI, "-L", BUILD,
                                     "-lcadise_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("cli build failed: %s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
