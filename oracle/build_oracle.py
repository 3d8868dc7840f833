"""Build recipe for the CPU oracle and reference harness (test infrastructure only).

* ``oracle/liboracle.so``: the C++ restatement of the reference path
  (trw_oracle.cpp), compiled with ``-ffp-contract=off``.
* ``oracle/_ref/ref_<app>``: the reference's own sampler code compiled from
  the reference tree with the Philox ``SFMT.h`` shim (ref_harness.cpp).  Built
  only where the reference tree exists; the binaries never leave this machine
  as source and are git-ignored.
* ``oracle/_ref/edgelist_to_csr``: the reference's EdgeList2CSR tool, same
  terms.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_APPS = ["deepwalk", "ppr", "node2vec", "metapath", "genericwalk"]


def _run(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("build failed: %s\n%s" % (" ".join(c), out.decode(errors="replace")))


def oracle_cmd():
    return ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
            os.path.join(HERE, "trw_oracle.cpp"), "-o", os.path.join(HERE, "liboracle.so")]


def ref_cmds(reference_root):
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    cmds = []
    for i, app in enumerate(REF_APPS):
        cmds.append(["g++", "-O2", "-std=c++14", "-ffp-contract=off", "-include", "cstdint", "-w",
                     "-DTRW_REF_APP=%d" % i,
                     "-I", os.path.join(HERE, "ref_shim"),
                     "-I", reference_root,
                     "-I", os.path.join(reference_root, "random_walk"),
                     os.path.join(HERE, "ref_harness.cpp"),
                     os.path.join(reference_root, "random_walk", "walker_generator.cpp"),
                     os.path.join(reference_root, "util", "graph", "graph.cpp"),
                     "-o", os.path.join(out_dir, "ref_" + app), "-pthread"])
    return cmds


def ref_tool_cmds(reference_root):
    """The reference's EdgeList2CSR tool (toolset/edgelist_to_csr.cpp over
    util/graph/graph.cpp), the oracle of thunderrw_gb300/toolset.py."""
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    return [["g++", "-O2", "-std=c++14", "-include", "cstdint", "-w", "-I", reference_root,
             os.path.join(reference_root, "toolset", "edgelist_to_csr.cpp"),
             os.path.join(reference_root, "util", "graph", "graph.cpp"),
             "-o", os.path.join(out_dir, "edgelist_to_csr"), "-pthread"]]


# Where this recipe reads the reference tree: the TRW_REFERENCE_ROOT
# environment variable, else the read-only mount of the build container.
# Machines without the tree (the GPU hosts) build the oracle alone.
REFERENCE_MOUNT = "/root/reference"


def reference_root_default():
    return os.environ.get("TRW_REFERENCE_ROOT") or REFERENCE_MOUNT


def build(reference_root=None, with_ref=True):
    reference_root = reference_root or reference_root_default()
    cmds = [oracle_cmd()]
    if with_ref and os.path.isdir(os.path.join(reference_root, "random_walk")):
        cmds += ref_cmds(reference_root) + ref_tool_cmds(reference_root)
    _run(cmds)


if __name__ == "__main__":
    build(*(sys.argv[1:2] or []))
