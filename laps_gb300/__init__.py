"""GB300 engine for LAPS's right-hand-side evaluation and RK3 time advance.

The compute path is hand-written CUDA for sm_103a in ``liblaps_gpu.so`` behind the C-ABI of
``include/laps_gpu.h``; ``laps_gb300.ffi`` binds it for Python hosts.  There is no CPU
fallback: without the library (or without a GPU) every compute call fails loudly.
"""
from .ffi import Laps, LapsError, load, params  # noqa: F401
from . import ffi  # noqa: F401
