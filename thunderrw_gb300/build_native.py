"""Builds libtrw_gpu.so in-tree from thunderrw_gb300/csrc/*.cu for sm_103a.

One nvcc process per translation unit, in parallel, then one link.  Every
unit is compiled with --fmad=false so each double operation of the sampling
and table-building arithmetic is a single IEEE round-to-nearest operation.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libtrw_gpu.so")
BUILD_DIR = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
              "-I", os.path.join(os.path.dirname(HERE), "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def build(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    objs, procs = [], []
    for src in sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
        if ptxas_verbose:
            cmd += ["-Xptxas", "-v"]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out.decode(errors="replace")))
        if verbose or ptxas_verbose:
            sys.stdout.write(out.decode(errors="replace"))
    link = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
    out = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if out.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (" ".join(link), out.stdout.decode(errors="replace")))
    return LIB


CLI_SRC = os.path.join(HERE, "cli", "trw_app.cpp")
BIN_DIR = os.path.join(HERE, "bin")
CLI_APPS = ["deepwalk", "ppr", "node2vec", "metapath", "genericwalk"]  # trw_app values 0..4


def build_cli() -> list:
    """The reference's app programs over libtrw_gpu.so: bin/<app>, one g++
    process per app, in parallel (host code only; no CUDA headers)."""
    os.makedirs(BIN_DIR, exist_ok=True)
    inc = os.path.join(os.path.dirname(HERE), "include")
    procs, outs = [], []
    for i, app in enumerate(CLI_APPS):
        out = os.path.join(BIN_DIR, app)
        cmd = [os.environ.get("CXX", "g++"), "-std=c++14", "-O2", "-Wall", "-DTRW_CLI_APP=%d" % i, "-I", inc,
               CLI_SRC, "-o", out, "-L", HERE, "-ltrw_gpu", "-Wl,-rpath,$ORIGIN/.."]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        outs.append(out)
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("g++ failed: %s\n%s" % (" ".join(cmd), out.decode(errors="replace")))
    return outs


if __name__ == "__main__":
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv))
    print("\n".join(build_cli()))
