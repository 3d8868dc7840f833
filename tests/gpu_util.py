"""Helpers shared by the GPU parity tests."""
import numpy as np
import pytest

from oracle import oracle as O


def need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from thunderrw_gb300 import engine as E
    E._lib()  # raises if the CUDA library is missing: no fallback
    return torch, E


def make_app(E, case):
    app = E.App(case["app"], case["mode"], case["sampler"], length=case["length"], p=case["p"], q=case["q"],
                tp=case["tp"], schema=case["schema"])
    return app


def oracle_run(g, case, sources, per_query=0, path_cap=None, counts=True):
    og = O.Graph(g["row"], g["adj"], g.get("weight"), g.get("label"))
    if case["mode"] == "static":
        og.build_tables(case["sampler"], 1 if case["app"] == "ppr" else 0)
    d = O.make_desc(case["app"], case["mode"], case["sampler"], length=case["length"], p=case["p"],
                    q=case["q"], tp=case["tp"], schema=case["schema"], seed=case["seed"])
    cap = path_cap if path_cap is not None else case["path_cap"]
    return og, O.walk(og, d, sources, per_query=per_query, id_base=case.get("id_base", 0), path_cap=cap,
                      want_counts=counts)


def to_np(t):
    return None if t is None else t.detach().cpu().numpy()
