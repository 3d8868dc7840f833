"""ctypes binding of libtrw_gpu.so (include/trw.h).

The library is built in-tree (thunderrw_gb300/libtrw_gpu.so, see
build_native.py).  There is no fallback: if the library is missing or fails to
load, importing the engine raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtrw_gpu.so")

TRW_OK = 0
ERRORS = {-1: "TRW_ERR_INVALID", -2: "TRW_ERR_CUDA", -3: "TRW_ERR_UNSUPPORTED", -4: "TRW_ERR_NO_TABLES",
          -5: "TRW_ERR_GRAPH", -6: "TRW_ERR_DEVICE", -7: "TRW_ERR_CAPACITY", -8: "TRW_ERR_BUSY"}

APPS = {"deepwalk": 0, "ppr": 1, "node2vec": 2, "metapath": 3, "genericwalk": 4}
MODES = {"uniform": 0, "static": 1, "dynamic": 2}
SAMPLERS = {"uniform": 0, "its": 1, "alias": 2, "rejection": 3, "maxweight_rejection": 4}
ENGINES = {"persistent": 0, "plain": 1}
WEIGHTS = {"edge": 0, "unit": 1}

EXPORTS = ["trw_graph_create", "trw_graph_destroy", "trw_graph_info", "trw_graph_synchronize", "trw_graph_indexes", "trw_graph_layout", "trw_graph_build_indexes", "trw_tables_build", "trw_tables_download", "trw_tables_upload",
           "trw_walk", "trw_ppr_batch", "trw_ppr_batch_sparse", "trw_set_engine_shape", "trw_get_engine_shape",
           "trw_profile_enable", "trw_profile_read", "trw_last_error",
           "trw_device_error", "trw_version"]


class TrwError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "TRW_ERR"), code, message))
        self.code = code


class WalkDesc(ctypes.Structure):
    _fields_ = [("app", ctypes.c_int32), ("mode", ctypes.c_int32), ("sampler", ctypes.c_int32),
                ("length", ctypes.c_int32), ("p", ctypes.c_double), ("q", ctypes.c_double),
                ("tp", ctypes.c_double), ("schema", ctypes.c_void_p), ("schema_len", ctypes.c_int32),
                ("seed", ctypes.c_uint64)]


_lib = None


def load(path: str = LIB_PATH):
    """Loads the CUDA library once; raises ImportError if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libtrw_gpu.so not built (run thunderrw_gb300/build_native.py or "
                          "__graft_entry__.build()); the engine has no CPU fallback")
    L = ctypes.CDLL(path)
    P, I32, I64, U32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32
    L.trw_graph_create.argtypes = [P, P, P, P, I32, I64, U32, ctypes.POINTER(P)]
    L.trw_graph_destroy.argtypes = [P]
    L.trw_graph_info.argtypes = [P, P, P, P]
    L.trw_graph_synchronize.argtypes = [P]
    L.trw_graph_indexes.argtypes = [P, P, P]
    L.trw_graph_layout.argtypes = [P, P, P]
    L.trw_graph_build_indexes.argtypes = [P, I32, I32, P]
    L.trw_tables_build.argtypes = [P, I32, I32, P]
    L.trw_tables_download.argtypes = [P, I32, P, ctypes.c_size_t]
    L.trw_tables_upload.argtypes = [P, I32, I32, P, ctypes.c_size_t, P]
    L.trw_walk.argtypes = [P, ctypes.POINTER(WalkDesc), P, I64, I64, P, I32, P, P, P, I32, P]
    L.trw_ppr_batch.argtypes = [P, ctypes.POINTER(WalkDesc), P, I64, I64, P, P, U32, I32, P]
    L.trw_ppr_batch_sparse.argtypes = [P, ctypes.POINTER(WalkDesc), P, I64, I64, P, P, P, I64, P, I32, P]
    L.trw_profile_enable.argtypes = [P, I32]
    L.trw_profile_read.argtypes = [P, P, P]
    L.trw_set_engine_shape.argtypes = [P, I32, I32, I32]
    L.trw_get_engine_shape.argtypes = [P, I32, P, P]
    L.trw_last_error.restype = ctypes.c_char_p
    L.trw_device_error.argtypes = [P, P]
    L.trw_version.restype = I32
    for name in EXPORTS:
        if name not in ("trw_last_error", "trw_version"):
            getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def check(rc: int):
    if rc != TRW_OK:
        msg = load().trw_last_error()
        raise TrwError(rc, msg.decode() if msg else "")
    return rc
