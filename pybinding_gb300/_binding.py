"""The engine's Python binding: the pybind11 module ``_kpm_gb300`` (``csrc/pykpm.cpp``).

A thin layer over the C ABI of ``include/kpm_gb300.h`` in the place of pybinding's own
pybind11 KPM module (``cppmodule/src/kpm.cpp``): ``Engine`` (one Hamiltonian or a ragged
batch), the KPM calculations as methods, NumPy arrays in and out, ``ValueError`` /
``RuntimeError`` as the reference raises them. The module is built in-tree next to
``libkpm_gb300.so`` and loaded from there; there is no other implementation to fall back on.
"""
from __future__ import annotations

import importlib.machinery
import importlib.util
import os
import threading

from . import build as _build

_lock = threading.Lock()
_module = None


def module():
    """Load (building first if needed) the extension module; ImportError if it cannot be."""
    global _module
    with _lock:
        if _module is None:
            path = _build.module_path()
            if not os.path.exists(path) or _build._stale():
                try:
                    _build.build()
                except Exception as e:  # no toolchain: the product cannot run
                    raise ImportError("pybinding_gb300: the engine module is missing and could not be built (%s). "
                                      "There is no CPU fallback." % e) from e
            loader = importlib.machinery.ExtensionFileLoader(_build.MODULE_NAME, path)
            spec = importlib.util.spec_from_file_location(_build.MODULE_NAME, path, loader=loader)
            mod = importlib.util.module_from_spec(spec)
            loader.exec_module(mod)
            _module = mod
        return _module


def Engine(hamiltonian, config=None, system_offsets=None):
    """An engine for ``hamiltonian`` (SciPy CSR, or anything ``csr_matrix`` accepts) with the
    configuration keywords of ``kpm()`` (``energy_range``, ``kernel``, ``kernel_param``,
    ``matrix_format``, ``optimal_size``, ``interleaved``, ``lanczos_precision``, ``precision``,
    ``batch_width``, ``tile_rows``, ``fuse_steps``, ``staging``)."""
    return module().Engine(hamiltonian, dict(config or {}), system_offsets)


def engine_batch(engines, config=None):
    """A ragged-batch engine whose system i is ``engines[i]``'s Hamiltonian (kpm_create_batch)."""
    return module().Engine.from_engines(list(engines), dict(config or {}))


def round_num_moments(n):
    return module().round_num_moments(int(n))


def damping_coefficients(kernel, param, num_moments):
    return module().damping_coefficients(kernel, float(param), int(num_moments))


def required_num_moments(kernel, param, scaled_broadening):
    return module().required_num_moments(kernel, float(param), float(scaled_broadening))
