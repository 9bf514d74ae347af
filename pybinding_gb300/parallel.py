"""Parameter sweeps: ``pb.parallelize`` / ``parallel_for`` / ``sweep`` / ``ndsweep``
(``pybinding/parallel.py:156-430``) with the GPU as the worker.

The reference runs each ``Deferred`` job of a sweep on its own CPU thread
(``parallel.py:29-70``). Here the jobs are produced first, then the deferred LDOS of
single-orbital models that share their settings (energies, broadening, kernel, scalar
type, engine options) run together: their Hamiltonians form one block-diagonal ragged
batch, and one recursion computes every model's LDOS, each model with its own spectral
bounds and moment count (``kpm_calc_ldos_batch``). Other jobs run one after another.
"""
from __future__ import annotations

import inspect
import itertools
import time
from copy import copy

import numpy as np

from . import _binding
from .chebyshev import DeferredLDOS
from .fileio import Versioned

__all__ = ["parallelize", "parallel_for", "sweep", "ndsweep", "Sweep", "NDSweep", "Factory"]

# rows of one batched recursion at most (bounded device memory per launch); larger groups
# are split into several batches
MAX_BATCH_ROWS = 1 << 26

# engine statistics (kpm_stats) of the last batched recursion and the host time of its two
# parts (assembling the batch, the engine call), for reports and benchmarks
last_batch_stats = None
last_batch_times = {}


class Factory:
    """Produces the deferred jobs of a sweep (``parallel.py:156-183``): ``sequence`` is the
    product of ``variables``; ``fixtures`` are the other parameters' defaults."""

    def __init__(self, variables, fixtures, produce):
        self.variables = variables
        self.fixtures = fixtures
        self.produce = produce
        self.sequence = list(itertools.product(*variables))


def parallelize(num_threads=None, queue_size=None, **kwargs):
    """Decorator making a :class:`Factory` from a function that returns a deferred job
    (``parallel.py:314-359``). ``num_threads`` and ``queue_size`` are accepted for
    compatibility; the GPU batches the jobs instead."""

    def decorator(produce_func):
        params = inspect.signature(produce_func).parameters
        variables = tuple(kwargs[k] for k in params if k in kwargs)
        fixtures = {k: v.default for k, v in params.items() if k not in kwargs}
        return Factory(variables, fixtures, produce_func)

    return decorator


def compute_all(deferred):
    """Compute every deferred job; deferred LDOS with equal :meth:`DeferredLDOS.batch_key`
    run as ragged batches (in their original order within a batch)."""
    groups, alone = {}, []
    for d in deferred:
        site = d.site if isinstance(d, DeferredLDOS) else None
        key = d.batch_key(site) if site is not None else None
        if key is None:
            alone.append(d)
        else:
            groups.setdefault(key, []).append((d, site))
    for members in groups.values():
        for chunk in _chunks(members):
            if len(chunk) == 1:
                chunk[0][0].compute()
            else:
                _run_ldos_batch(chunk)
    for d in alone:
        d.compute()


def _chunks(members):
    chunk, rows = [], 0
    for d, site in members:
        n = d.impl.model.hamiltonian.shape[0]
        if chunk and rows + n > MAX_BATCH_ROWS:
            yield chunk
            chunk, rows = [], 0
        chunk.append((d, site))
        rows += n
    if chunk:
        yield chunk


def _run_ldos_batch(chunk):
    """Run the (job, site) pairs of ``chunk`` as one ragged batch."""
    global last_batch_stats, last_batch_times
    sites = [site for _, site in chunk]
    chunk = [d for d, _ in chunk]
    first = chunk[0].impl
    t0 = time.perf_counter()
    # the jobs' own engines already hold their checked matrices: concatenate those
    engine = _binding.engine_batch([d.impl.engine for d in chunk], first._cfg_args)
    t1 = time.perf_counter()
    try:
        out = engine.calc_ldos_batch(sites, chunk[0].energy, chunk[0].broadening)
        last_batch_stats = engine.stats()
    finally:
        engine.close()
    last_batch_times = dict(assemble_s=t1 - t0, call_s=time.perf_counter() - t1)
    for d, ldos in zip(chunk, out):
        d.result = ldos[:, None]  # (energies, orbitals), as calc_ldos returns it


def parallel_for(factory, make_result=None):
    """Run every job of ``factory`` and return ``make_result(data)`` (or the list of
    results), ``data`` holding one result per value of ``factory.sequence``
    (``parallel.py:282-311``)."""
    jobs = [factory.produce(*var, **factory.fixtures) for var in factory.sequence]
    compute_all(jobs)
    data = [copy(d.result) for d in jobs]
    return make_result(data) if make_result else data


class Sweep(Versioned):
    """2D parameter sweep result (``pybinding/results.py:772-800``): ``data[i, j]`` at
    ``x[i]``, ``y[j]``."""

    def __init__(self, x, y, data, labels=None, tags=None):
        self.x = np.atleast_1d(x)
        self.y = np.atleast_1d(y)
        self.data = np.atleast_2d(data)
        self.labels = dict(dict(title="", x="x", y="y", data="data"), **(labels or {}))
        self.tags = tags


class NDSweep(Versioned):
    """N-dimensional sweep result (``pybinding/results.py:1027-1052``)."""

    def __init__(self, variables, data, labels=None, tags=None):
        self.variables = variables
        self.data = np.reshape(data, [len(v) for v in variables])
        self.labels = dict(dict(title="", axes=[], data="data"), **(labels or {}))
        for axis, label in zip("xyz", self.labels["axes"]):
            self.labels[axis] = label
        self.tags = tags


def sweep(factory, plot=None, labels=None, tags=None, silent=False):
    """Sweep over the first variable; ``energy`` is the factory's fixture (``parallel.py:362-393``)."""
    x = factory.variables[0]
    energy = factory.fixtures["energy"]
    zero = np.zeros_like(energy, np.float32)

    def make_result(data):
        return Sweep(x, energy, np.vstack([v.squeeze() if v is not None else zero for v in data]), labels, tags)

    return parallel_for(factory, make_result)


def ndsweep(factory, plot=None, labels=None, tags=None, silent=False):
    """Sweep over every variable and the ``energy`` fixture (``parallel.py:396-430``)."""
    energy = factory.fixtures["energy"]
    variables = factory.variables + (energy,)
    zero = np.zeros_like(energy, np.float32)

    def make_result(data):
        return NDSweep(variables, np.vstack([v.squeeze() if v is not None else zero for v in data]), labels, tags)

    return parallel_for(factory, make_result)
