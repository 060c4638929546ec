"""nhwave_gb300 -- GB300 (sm_103a) implementation of NHWAVE's time-step hot path.

The compute path is ``libnhw_gpu.so`` (hand-written CUDA kernels behind the
C-ABI of ``include/nhwave_gb300.h``); this package holds its ctypes binding
(:mod:`.lib`), the run-time parameters (:mod:`.params`, including an
``input.txt`` reader), field ids (:mod:`.fields`), seeded synthetic scenarios
(:mod:`.scenarios`) and the in-tree build (:mod:`.build`).
"""
from . import fields, params, scenarios  # noqa: F401
from .params import NhwParams, NhwScalars, default_params, read_input  # noqa: F401

__all__ = ["fields", "params", "scenarios", "NhwParams", "NhwScalars", "default_params", "read_input"]
