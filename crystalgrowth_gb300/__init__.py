"""crystalgrowth_gb300 -- the Kobayashi dendritic-growth phase-field step of
jklae/CrystalGrowth (src/Kobayashi.cpp), rebuilt for one GB300 (sm_103a) in
FP64 behind a C ABI (include/kobayashi_gpu.h).

The compute path is libkobayashi_gpu.so (hand-written CUDA); this package is a
thin ctypes front end used by the tests and the benchmark.  There is no CPU
fallback: every call fails loudly if the library is missing.
"""
from ._lib import KgError, lib, load, Params  # noqa: F401
from .kobayashi import Kobayashi  # noqa: F401
from .batch import Batch  # noqa: F401
from .adjoint import Adjoint  # noqa: F401
from . import configs  # noqa: F401

__all__ = ["Adjoint", "Batch", "Kobayashi", "KgError", "Params", "configs", "lib", "load"]
