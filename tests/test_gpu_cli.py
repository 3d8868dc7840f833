"""The reference-style app programs (thunderrw_gb300/bin/<app>) on the GPU:
each run's paths and lengths (written with -o) equal the oracle's walks from
the same sources, and the reported step count is the oracle's."""
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import need_gpu

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "thunderrw_gb300", "bin")


@pytest.fixture(scope="module")
def graph_dir(tmp_path_factory):
    need_gpu()
    from thunderrw_gb300 import build_native, formats
    from thunderrw_gb300 import generators as G
    if not os.path.exists(os.path.join(BIN, "genericwalk")):
        build_native.build_cli()
    g = G.make_graph("rmat", 1 << 11, 12, seed=17, labels=4)
    d = tmp_path_factory.mktemp("graph")
    formats.store_csr(str(d), g["row"], g["adj"], weight=g["weight"], label=g["label"])
    og = O.Graph(g["row"], g["adj"], g["weight"], g["label"])
    return str(d), og


def _run(app, args, prefix):
    r = subprocess.run([os.path.join(BIN, app)] + args + ["-o", prefix], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    steps = int(re.search(r"Num of steps: (\d+)", r.stdout).group(1))
    paths = np.fromfile(prefix + ".paths.bin", dtype=np.int32)
    lengths = np.fromfile(prefix + ".lengths.bin", dtype=np.int32)
    return steps, paths.reshape(lengths.size, -1), lengths, r.stdout


@pytest.mark.parametrize("app,args,desc", [
    ("deepwalk", ["-ew", "-l", "15"], ("deepwalk", "static", "alias", dict(length=15))),
    ("ppr", ["-sp", "0.25", "-nw", "3000"], ("ppr", "uniform", "uniform", dict(length=1, tp=0.25))),
    ("node2vec", ["-l", "12", "-p", "0.3", "-q", "3"],
     ("node2vec", "dynamic", "maxweight_rejection",
      dict(length=12, p=float(np.float32(0.3)), q=float(np.float32(3.0))))),
    ("metapath", ["-el", "-l", "10", "-s", "0,1,3"], ("metapath", "dynamic", "its", dict(length=10, schema=[0, 1, 3]))),
    ("genericwalk", ["-ew", "-l", "9", "-st", "2", "-wn", "500", "-seed", "7"],
     ("genericwalk", "static", "its", dict(length=9, seed=7))),
    ("genericwalk", ["-ew", "-l", "9", "-em", "2", "-sm", "2"], ("genericwalk", "dynamic", "alias", dict(length=9))),
])
def test_cli_matches_oracle(graph_dir, tmp_path, app, args, desc):
    d, og = graph_dir
    steps, paths, lengths, out = _run(app, ["-f", d, "-n", "4"] + args, str(tmp_path / "out"))
    name, mode, sampler, kw = desc
    if mode == "static":
        og.build_tables(sampler, 1 if name == "ppr" else 0)
    src = paths[:, 0].copy()
    assert np.all(np.diff(og.row)[src] > 0)  # every generator skips isolated vertices
    cap = paths.shape[1]
    kw = dict(kw)
    seed = kw.pop("seed", 1)
    ref = O.walk(og, O.make_desc(name, mode, sampler, seed=seed, **kw), src, path_cap=cap)
    assert steps == ref["steps"]
    np.testing.assert_array_equal(lengths, ref["lengths"])
    np.testing.assert_array_equal(paths, ref["paths"])
    if app == "ppr":
        hub = int(np.argmax(np.diff(og.row)))
        assert np.all(src == hub) and src.size == 3000


@pytest.mark.parametrize("flag,sampler,sm", [("-al", "alias", "2"), ("-ep", "its", "1"), ("-rj", "rejection", "3")])
def test_cli_loads_precomputed_tables(graph_dir, tmp_path, flag, sampler, sm):
    """-al / -ep / -rj read the reference's table files (written here from the
    oracle's builders, byte-identical to the reference preprocessors' output)
    and the static walk uses them instead of building its own; the walks are
    the oracle's, and no initialization (table build) is logged."""
    from thunderrw_gb300 import formats
    d, og = graph_dir
    tdir = tmp_path / "tables"
    og.build_tables(sampler, 0)
    kw = {"alias": dict(alias=og.alias), "its": dict(prefix=og.prefix), "rejection": dict(rmax=og.rej_max)}[sampler]
    formats.store_csr(str(tdir), og.row, og.adj, weight=og.weight, label=og.label, **kw)
    steps, paths, lengths, out = _run("deepwalk", ["-f", str(tdir), "-ew", flag, "-em", "1", "-sm", sm, "-l", "11"],
                                      str(tmp_path / "out"))
    assert "Loaded tables" in out and "Initialization time" not in out
    ref = O.walk(og, O.make_desc("deepwalk", "static", sampler, length=11, seed=1), paths[:, 0].copy(), path_cap=11)
    assert steps == ref["steps"]
    np.testing.assert_array_equal(paths, ref["paths"])


def test_upload_table_round_trip():
    """A table downloaded from one graph and uploaded into another copy of it
    gives the same walks as building it there; a wrong size is refused."""
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import generators as G
    g = G.make_graph("chunglu", 1 << 12, 10, seed=5)
    a = E.Graph(g["row"], g["adj"], g["weight"])
    b = E.Graph(g["row"], g["adj"], g["weight"])
    try:
        a.build_tables("alias", "edge")
        tab = a.download_table("alias")
        b.upload_table("alias", tab)
        assert b.download_table("alias").tobytes() == tab.tobytes()
        src = G.all_sources(g["row"], seed=2)[:1500]
        ra = E.compute(a, src, E.DeepWalk(20), seed=3)
        rb = E.compute(b, src, E.DeepWalk(20), seed=3)
        assert torch.equal(ra.paths, rb.paths) and ra.steps == rb.steps
        with pytest.raises(N.TrwError):
            b.upload_table("alias", tab[:-1])
    finally:
        a.close()
        b.close()
