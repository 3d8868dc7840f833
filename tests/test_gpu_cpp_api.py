"""The C++ mirror of the reference interface (include/trw.hpp): a program
written like a ThunderRW app (load_csr, generate_all_source, compute<App>)
links libtrw_gpu.so and walks exactly what the oracle walks."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import need_gpu

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _fnv(paths, lengths):
    h = 1469598103934665603
    for x in list(paths.ravel()) + list(lengths.ravel()):
        h = ((h ^ (int(x) & 0xFFFFFFFF)) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    need_gpu()
    if not shutil.which("g++"):
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("cpp") / "hpp_walk")
    lib_dir = os.path.join(ROOT, "thunderrw_gb300")
    subprocess.run(["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "hpp_walk.cpp"), "-L", lib_dir, "-ltrw_gpu",
                    "-Wl,-rpath," + lib_dir, "-o", out], check=True)
    return out


@pytest.mark.parametrize("app,mode,sampler", [("deepwalk", "static", "alias"),
                                              ("node2vec", "dynamic", "maxweight_rejection"),
                                              ("metapath", "dynamic", "its"), ("ppr", "uniform", "uniform")])
def test_cpp_compute_matches_oracle(exe, tmp_path, app, mode, sampler):
    from thunderrw_gb300 import formats
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 10, 10, seed=13, labels=5)
    formats.store_csr(str(tmp_path), g["row"], g["adj"], weight=g["weight"], label=g["label"])
    out = subprocess.run([exe, str(tmp_path), app], check=True, capture_output=True, text=True).stdout.split()
    pre = subprocess.run([exe, str(tmp_path), app, "prebuilt"], check=True, capture_output=True, text=True).stdout.split()
    assert pre == out  # lookup structures built up front: the same walks
    og = O.Graph(g["row"], g["adj"], g["weight"], g["label"])
    if mode == "static":
        og.build_tables(sampler, 0)
    cap = 1 if app == "ppr" else 20
    src = np.nonzero(np.diff(og.row))[0].astype(np.int32)  # generate_all_source without shuffle
    d = O.make_desc(app, mode, sampler, length=20, p=2.0, q=0.5, tp=0.2, schema=[0, 1, 2, 3, 4], seed=1)
    ref = O.walk(og, d, src, path_cap=cap)
    assert int(out[0]) == ref["steps"]
    assert int(out[1]) == _fnv(ref["paths"], ref["lengths"])
