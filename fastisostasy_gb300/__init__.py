"""GB300-native LV-ELVA glacial-isostatic-adjustment path of FastIsostasy.

The compute lives in ``libfigpu.so`` (hand-written sm_103a CUDA kernels behind
the C ABI of ``include/fi_gpu.h``); this package holds the build recipe, the
ctypes binding, the host-side mirror of the reference's Fortran API and the
synthetic workloads.
"""
from . import params, workloads  # noqa: F401

__all__ = ["params", "workloads", "isostasy", "build"]
