"""GB300-native random-walk engine with ThunderRW's step-centric API.

The walk path runs in libtrw_gpu.so (hand-written sm_103a CUDA behind the C
ABI of include/trw.h); ``thunderrw_gb300.engine`` is its Python host side and
needs that library.  ``generators`` and ``formats`` are plain data tools.
"""
from . import formats, generators  # noqa: F401
