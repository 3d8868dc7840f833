"""Loader for the golden fixtures produced by tests/golden/make_golden.py
(outputs of the reference's own sampler code under the Philox shim)."""
import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

with open(os.path.join(HERE, "manifest.json")) as _f:
    MANIFEST = json.load(_f)
_GRAPHS = np.load(os.path.join(HERE, "graphs.npz"))
_CASES = np.load(os.path.join(HERE, "cases.npz"))

CASES = MANIFEST["cases"]
PHILOX_KAT = MANIFEST["philox_kat"]


def graph_arrays(name):
    return {k: _GRAPHS[name + "/" + k] for k in ("row", "adj", "weight", "label")}


def case_arrays(case):
    key = case["key"]
    return {k.split("/", 1)[1]: _CASES[k] for k in _CASES.files if k.startswith(key + "/")}


def case_id(case):
    return "%s-%s-%s-%s-%s" % (case["key"], case["graph"], case["app"], case["mode"], case["sampler"])
