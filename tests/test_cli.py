"""The reference-style app programs (thunderrw_gb300/bin/<app>): flag
handling that needs no GPU.  Runs on the GPU are in test_gpu_cli.py."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "thunderrw_gb300", "bin")
APPS = ["deepwalk", "ppr", "node2vec", "metapath", "genericwalk"]


@pytest.fixture(scope="module")
def bins():
    if not all(os.path.exists(os.path.join(BIN, a)) for a in APPS):
        if not os.path.exists(os.path.join(ROOT, "thunderrw_gb300", "libtrw_gpu.so")):
            pytest.skip("libtrw_gpu.so not built")
        from thunderrw_gb300 import build_native
        build_native.build_cli()
    return {a: os.path.join(BIN, a) for a in APPS}


@pytest.mark.parametrize("app", APPS)
def test_usage_without_graph(bins, app):
    r = subprocess.run([bins[app]], capture_output=True, text=True)
    assert r.returncode == 2 and "usage: %s -f <graph dir>" % app in r.stderr
    r = subprocess.run([bins[app], "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "app flags" in r.stderr


@pytest.mark.parametrize("app", APPS)
def test_missing_graph_files(bins, app, tmp_path):
    r = subprocess.run([bins[app], "-f", str(tmp_path / "none"), "-ew"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr and "b_degree.bin" in r.stderr
