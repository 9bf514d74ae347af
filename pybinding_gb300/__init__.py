"""pybinding_gb300: a GB300-native kernel polynomial method (KPM) engine.

A drop-in backend for pybinding's ``pb.kpm(model, ...) -> KPM`` path. The
computation runs in hand-written CUDA kernels for sm_103a behind a C ABI
(``include/kpm_gb300.h``); this package holds the Python side of that
boundary. There is no CPU fallback: calls fail if the CUDA library cannot be
loaded or no GPU is present.
"""
from . import adjoint
from .fileio import load, save
from .parallel import NDSweep, Sweep, ndsweep, parallel_for, parallelize, sweep
from .chebyshev import (KPM, KPMBatch, Series, SpatialLDOS, dirichlet_kernel, jackson_kernel, kpm, kpm_batch,
                        lorentz_kernel)

__all__ = ["KPM", "KPMBatch", "Series", "SpatialLDOS", "kpm", "kpm_batch", "jackson_kernel", "lorentz_kernel",
           "dirichlet_kernel", "adjoint", "save", "load", "parallelize", "parallel_for", "sweep", "ndsweep",
           "Sweep", "NDSweep"]
