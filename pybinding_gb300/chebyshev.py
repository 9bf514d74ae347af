"""The ``pb.kpm`` interface backed by the GB300 engine.

Mirrors ``pybinding/chebyshev.py``: :class:`KPM` is the same thin wrapper over
an ``impl`` object, :func:`kpm` mirrors ``pb.kpm`` / ``_cpp.kpm``
(``cppmodule/src/kpm.cpp:8-37``) and the kernels mirror
``jackson_kernel`` / ``lorentz_kernel`` / ``dirichlet_kernel``. The ``impl``
here, :class:`GpuImpl`, has the methods and properties that
``chebyshev.KPM`` calls on ``_cpp.KPM``; every computation runs in the CUDA
engine through the C ABI (``include/kpm_gb300.h``).

A model is duck-typed: anything with ``.hamiltonian`` (a SciPy CSR matrix) and
``.system`` (``positions``, ``find_nearest``, ``to_hamiltonian_indices``,
``sublattice_range``) works, including :class:`pybinding_gb300.lattice.Model`.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import _binding
from .fileio import Versioned

__all__ = ["KPM", "kpm", "kpm_batch", "jackson_kernel", "lorentz_kernel", "dirichlet_kernel", "Series",
           "SpatialLDOS", "KPMBatch", "ComputeProgressReporter"]


class Series(Versioned):
    """A 1D (or column-wise 2D) data series over a variable: the part of
    ``pybinding.results.Series`` (``pybinding/results.py:162-215``) that KPM returns."""

    def __init__(self, variable, data, labels=None):
        self.variable = np.atleast_1d(variable)
        self.data = np.atleast_1d(data)
        self.labels = dict(variable="x", data="y", columns="") if labels is None else labels

    def with_data(self, data):
        return Series(self.variable, data, self.labels)

    def reduced(self):
        return self.with_data(self.data.sum(axis=1)) if self.data.ndim > 1 else self

    def __repr__(self):
        return "Series(%s -> %s, %d points)" % (self.labels.get("variable"), self.labels.get("data"),
                                               self.variable.size)


class SpatialLDOS:
    """Result of :meth:`KPM.calc_spatial_ldos` (``pybinding/chebyshev.py:22-62``)."""

    def __init__(self, data, energy, indices, positions):
        self.data = data
        self.energy = energy
        self.indices = indices
        self.positions = positions

    def ldos(self, position):
        x, y, z = self.positions
        p = np.zeros(3, np.float32)
        pos = np.asarray(position, np.float32).ravel()
        p[:pos.size] = pos
        i = int(np.argmin((x - p[0]) ** 2 + (y - p[1]) ** 2 + (z - p[2]) ** 2))
        return Series(self.energy, self.data[:, i], labels=dict(variable="E (eV)", data="LDOS", columns="orbitals"))

    def structure_map(self, energy):
        idx = int(np.argmin(abs(self.energy - energy)))
        return self.positions, self.data[idx]


class Kernel:
    """Damping kernel: ``KPMKernel`` (``cppmodule/src/kpm.cpp:68-74``, ``kpm/Kernel.cpp:6-50``)."""

    def __init__(self, name, param=4.0):
        if name == "lorentz" and param <= 0:
            raise ValueError("Lorentz kernel: lambda must be positive.")
        self.name = name
        self.param = float(param)

    def damping_coefficients(self, num_moments):
        return _binding.damping_coefficients(self.name, self.param, num_moments)

    def required_num_moments(self, scaled_broadening):
        return _binding.required_num_moments(self.name, self.param, scaled_broadening)

    def __repr__(self):
        return "%s_kernel(%s)" % (self.name, "" if self.name != "lorentz" else self.param)


def jackson_kernel():
    """The Jackson kernel: Gaussian broadening ``sigma = pi / N``."""
    return Kernel("jackson")


def lorentz_kernel(lambda_value=4.0):
    """The Lorentz kernel: Lorentzian broadening ``lambda / N``; best for Green's functions."""
    return Kernel("lorentz", lambda_value)


def dirichlet_kernel():
    """The Dirichlet kernel: raw (undamped) moments."""
    return Kernel("dirichlet")


class KPMStats:
    """``KPMStats`` (``cppmodule/src/kpm.cpp:50-66``) from the engine's ``kpm_stats``."""

    def __init__(self, s):
        self.__dict__.update(vars(s))
        self.uses_full_system = bool(self.uses_full_system)


def _dtype_of(model):
    return np.dtype(sp.csr_matrix(model.hamiltonian).dtype)


def _is_multiorbital(model):
    """``Model::is_multiorbital``: more Hamiltonian rows than sites (duck-typed models that do not
    say so themselves are judged by their system's sizes)."""
    flag = getattr(model, "is_multiorbital", None)
    if flag is not None:
        return bool(flag() if callable(flag) else flag)
    system = getattr(model, "system", None)
    size = getattr(system, "hamiltonian_size", None)
    sites = getattr(system, "num_sites", None)
    return size is not None and sites is not None and size != sites


class GpuImpl:
    """The ``impl`` object of :class:`KPM`: ``_cpp.KPM`` semantics on the CUDA engine."""

    def __init__(self, model, energy_range=(0, 0), kernel=None, matrix_format="ELL", optimal_size=True,
                 interleaved=True, lanczos_precision=0.002, precision="auto", batch_width=0, tile_rows=0,
                 moments_gemm="fp64", staging="auto", num_threads="auto", progress_callback=None, **_):
        if moments_gemm not in ("fp64", "tensor"):
            raise ValueError("moments_gemm must be 'fp64' or 'tensor'")
        self.kernel = kernel if kernel is not None else jackson_kernel()
        self._gemm_mode = 1 if moments_gemm == "tensor" else 0
        self._cfg_args = dict(energy_range=tuple(energy_range), kernel=self.kernel.name,
                              kernel_param=self.kernel.param, matrix_format=matrix_format,
                              optimal_size=optimal_size, interleaved=interleaved,
                              lanczos_precision=lanczos_precision, precision=precision, batch_width=batch_width,
                              tile_rows=tile_rows, staging=staging,
                              num_threads=0 if num_threads in (None, "auto") else int(num_threads))
        self._model = model
        self._engine = _binding.Engine(model.hamiltonian, self._cfg_args)
        if progress_callback is not None:
            self._engine.set_progress_callback(progress_callback)

    # -------------------------------------------------------------- properties
    @property
    def model(self):
        return self._model

    @model.setter
    def model(self, model):
        self._model = model
        self._engine.set_hamiltonian(model.hamiltonian)

    @property
    def system(self):
        return self._model.system

    @property
    def scaling_factors(self):
        return self._engine.scaling_factors(0)

    @property
    def energy_bounds(self):
        return self._engine.energy_bounds(0)[:2]

    @property
    def stats(self):
        return KPMStats(self._engine.stats())

    @property
    def engine(self):
        return self._engine

    def report(self, shortform=False):
        return self._engine.report(shortform)

    # -------------------------------------------------------------- calculations
    def moments(self, num_moments, alpha, beta, op):
        """``KPM::moments`` (cppcore/src/KPM.cpp:19-53)"""
        alpha = np.atleast_1d(np.asarray(alpha))
        beta = np.asarray(beta) if beta is not None else np.array([])
        return self._engine.moments(num_moments, alpha, beta, op)

    def calc_greens(self, i, j, energy, broadening):
        """``KPM::calc_greens`` (KPM.cpp:103-129): one element, or a list for a list of columns."""
        if np.ndim(j) == 0:
            return self._engine.calc_greens(i, [j], energy, broadening)[0]
        return list(self._engine.calc_greens(i, list(j), energy, broadening))

    def calc_ldos(self, energy, broadening, position, sublattice="", reduce=True):
        """``KPM::calc_ldos`` (KPM.cpp:55-65): nearest site, all its orbitals."""
        system = self._model.system
        site = system.find_nearest(position, sublattice)
        idx = np.atleast_1d(system.to_hamiltonian_indices(site))
        ldos = self._engine.calc_ldos(idx, energy, broadening)
        if reduce and ldos.shape[1] > 1:
            return ldos.sum(axis=1)
        return ldos

    def calc_spatial_ldos(self, energy, broadening, shape, sublattice=""):
        """``KPM::calc_spatial_ldos`` (KPM.cpp:67-94): every site inside ``shape``, single-orbital
        models only (site index = Hamiltonian index), like the reference."""
        if _is_multiorbital(self._model):
            raise RuntimeError("This function doesn't currently support multi-orbital models")
        system = self._model.system
        x, y, z = system.positions
        contains = shape(x, y, z) if callable(shape) else shape.contains(x, y, z)
        start, end = system.sublattice_range(sublattice)
        mask = np.zeros(x.size, bool)
        mask[start:end] = np.asarray(contains, bool)[start:end]
        idx = np.nonzero(mask)[0]
        if idx.size == 0:
            return np.zeros((np.size(energy), 0))
        return self._engine.calc_ldos(idx, energy, broadening)

    def calc_dos(self, energy, broadening, num_random):
        """``KPM::calc_dos`` (KPM.cpp:96-101)"""
        return self._engine.calc_dos(energy, broadening, num_random)[0]

    def deferred_ldos(self, energy, broadening, position, sublattice=""):
        """``deferred_ldos`` (cppmodule/src/kpm.cpp:84-91): compute on demand."""
        return DeferredLDOS(self, energy, broadening, position, sublattice)

    def calc_conductivity(self, chemical_potential, broadening, temperature, direction, num_random, num_points,
                          gemm_mode=None):
        """``KPM::calc_conductivity`` (KPM.cpp:131-149); returns the real part."""
        if len(direction) != 2 or any(c not in "xyz" for c in direction):
            raise RuntimeError("Invalid direction: must be 'xx', 'xy', 'zz', or similar.")
        if gemm_mode is None:
            gemm_mode = self._gemm_mode
        pos = dict(zip("xyz", self._model.system.positions))
        out = self._engine.calc_conductivity(pos[direction[0]], pos[direction[1]], chemical_potential, broadening,
                                             temperature, num_random, num_points, gemm_mode)
        return out.real


class Deferred:
    """A computation run by :meth:`compute`, result in :attr:`result` (``cppmodule/include/thread.hpp``)."""

    def __init__(self, fn):
        self._fn = fn
        self.result = None

    def compute(self):
        self.result = self._fn()
        return self.result


class DeferredLDOS(Deferred):
    """``KPM.deferred_ldos`` (``cppmodule/src/kpm.cpp:84-91``): the LDOS of one model at the
    site nearest to ``position``, computed on demand. :func:`pybinding_gb300.parallel.parallel_for`
    runs the deferred LDOS of many single-orbital models together, as one ragged batch."""

    def __init__(self, impl, energy, broadening, position, sublattice=""):
        super().__init__(lambda: impl.calc_ldos(energy, broadening, position, sublattice))
        self.impl = impl
        self.energy = np.asarray(energy, dtype=np.float64)
        self.broadening = float(broadening)
        self.position = position
        self.sublattice = sublattice

    @property
    def site(self):
        """Hamiltonian row of the site nearest to ``position`` in the model as it is now (as
        ``calc_ldos`` finds it when the job runs); None for a multi-orbital site."""
        system = self.impl.model.system
        idx = np.atleast_1d(system.to_hamiltonian_indices(system.find_nearest(self.position, self.sublattice)))
        return int(idx[0]) if idx.size == 1 else None

    def batch_key(self, site=None):
        """Deferred LDOS with equal keys can share one recursion (None: this one cannot, e.g. a
        multi-orbital site). ``site``: the job's :attr:`site`, when already known."""
        if (self.site if site is None else site) is None:
            return None
        cfg = tuple(sorted((k, v) for k, v in self.impl._cfg_args.items()))
        return (cfg, np.dtype(self.impl.model.hamiltonian.dtype).str, self.energy.tobytes(), self.broadening)


class KPM:
    """The common interface of KPM implementations (``pybinding/chebyshev.py:65-317``)."""

    def __init__(self, impl):
        if hasattr(impl, "hamiltonian") and hasattr(impl, "system") and not hasattr(impl, "calc_dos"):
            raise TypeError("You're probably looking for `pb.kpm()` (lowercase).")
        self.impl = impl

    @property
    def model(self):
        return self.impl.model

    @model.setter
    def model(self, model):
        self.impl.model = model

    @property
    def system(self):
        return self.impl.system

    @property
    def scaling_factors(self):
        return self.impl.scaling_factors

    @property
    def kernel(self):
        return self.impl.kernel

    @property
    def stats(self):
        return self.impl.stats

    def report(self, shortform=False):
        return self.impl.report(shortform)

    def moments(self, num_moments, alpha, beta=None, op=None):
        """mu_n = <beta| op T_n(H) |alpha> (chebyshev.py:117-149)"""
        if beta is None:
            beta = []
        if op is None:
            op = sp.csr_matrix((0, 0))
        else:
            op = sp.csr_matrix(op)
        return self.impl.moments(num_moments, alpha, beta, op)

    def calc_greens(self, i, j, energy, broadening):
        return self.impl.calc_greens(i, j, energy, broadening)

    def calc_ldos(self, energy, broadening, position, sublattice="", reduce=True):
        ldos = self.impl.calc_ldos(energy, broadening, position, sublattice, reduce)
        return Series(energy, np.squeeze(ldos), labels=dict(variable="E (eV)", data="LDOS", columns="orbitals"))

    def calc_spatial_ldos(self, energy, broadening, shape, sublattice=""):
        ldos = self.impl.calc_spatial_ldos(energy, broadening, shape, sublattice)
        system = self.impl.system
        x, y, z = system.positions
        contains = shape(x, y, z) if callable(shape) else shape.contains(x, y, z)
        start, end = system.sublattice_range(sublattice)
        mask = np.zeros(x.size, bool)
        mask[start:end] = np.asarray(contains, bool)[start:end]
        idx = np.nonzero(mask)[0]
        return SpatialLDOS(ldos, energy, idx, (x[idx], y[idx], z[idx]))

    def calc_dos(self, energy, broadening, num_random=1):
        dos = self.impl.calc_dos(energy, broadening, num_random)
        return Series(energy, dos, labels=dict(variable="E (eV)", data="DOS"))

    def deferred_ldos(self, energy, broadening, position, sublattice=""):
        return self.impl.deferred_ldos(energy, broadening, position, sublattice)

    def calc_conductivity(self, chemical_potential, broadening, temperature, direction="xx", volume=1.0,
                          num_random=1, num_points=1000):
        data = self.impl.calc_conductivity(chemical_potential, broadening, temperature, direction, num_random,
                                           num_points)
        if volume != 1.0:
            data = data / volume
        return Series(chemical_potential, data, labels=dict(variable=r"$\mu$ (eV)", data=r"$\sigma (e^2/h)$"))


class ComputeProgressReporter:
    """The default progress callback of :func:`kpm` (``pybinding/chebyshev.py:320-336``): prints
    when the moments of a DOS start, then the share of the vectors done."""

    def __init__(self, stream=None):
        self.stream = stream
        self.done = 0

    def _print(self, text, end="\n"):
        import sys
        out = self.stream or sys.stdout
        out.write(text + end)
        out.flush()

    def __call__(self, delta, total):
        if total == 1:
            return  # short jobs are not reported
        if delta < 0:  # start
            self.done = 0
            self._print("Computing KPM moments...")
        elif delta == total:  # finish (increments are smaller than the total)
            self._print("\r100%")
        else:
            self.done += delta
            self._print("\r%3d%%" % (100 * self.done // total), end="")


def kpm(model, energy_range=None, kernel="default", num_threads="auto", silent=False, **kwargs):
    """GB300 KPM for ``model`` -- same signature as ``pb.kpm`` (pybinding/chebyshev.py:339-378).

    Extra keyword arguments of ``_cpp.kpm`` are accepted: ``matrix_format``,
    ``optimal_size``, ``interleaved``, ``lanczos_precision``; plus the GPU knobs
    ``precision`` ("auto"; "fp64"; FP32 vectors with row sums of chained FMAs "fp32", compensated
    by one FMA per term "fp32p" -- the automatic choice for a float32 H -- or by TwoSum "fp32x"),
    ``batch_width`` and ``moments_gemm``
    ("fp64": the conductivity's moments matrix on the FP64 CUDA cores; "tensor": on
    the tensor cores from FP32 planes, three-product TF32 split). ``num_threads`` is the
    number of host threads for the engine's setup work (the recursion runs on the GPU).
    ``progress_callback(delta, total)`` follows the reference's protocol during ``calc_dos``
    (a :class:`ComputeProgressReporter` unless ``silent``).
    """
    if kernel == "default":
        kernel = jackson_kernel()
    if "progress_callback" not in kwargs:
        kwargs["progress_callback"] = ComputeProgressReporter()
    if silent:
        kwargs["progress_callback"] = None
    return KPM(GpuImpl(model, energy_range or (0, 0), kernel, num_threads=num_threads, **kwargs))


def block_diagonal(hs):
    """The block-diagonal CSR matrix of square CSR matrices ``hs`` (sorted indices, int32),
    in their common scalar type: their index arrays shifted and concatenated."""
    dt = np.result_type(*[h.dtype for h in hs])
    rows = np.concatenate([[0], np.cumsum([h.shape[0] for h in hs])]).astype(np.int64)
    nnz = np.concatenate([[0], np.cumsum([h.nnz for h in hs])]).astype(np.int64)
    if rows[-1] >= 2 ** 31 or nnz[-1] >= 2 ** 31:
        raise ValueError("the batch exceeds int32 indices")
    parts = []
    for h in hs:
        if h.shape[0] != h.shape[1]:
            raise ValueError("Hamiltonians must be square")
        h = h.copy() if not h.has_sorted_indices else h
        h.sort_indices()
        parts.append(h)
    # int32 arithmetic: every sum is below the 2^31 checked above
    indptr = np.empty(int(rows[-1]) + 1, np.int32)
    indices = np.empty(int(nnz[-1]), np.int32)
    data = np.empty(int(nnz[-1]), dt)
    indptr[0] = 0
    for i, p in enumerate(parts):
        np.add(p.indptr[1:], np.int32(nnz[i]), out=indptr[rows[i] + 1:rows[i + 1] + 1], dtype=np.int32, casting="unsafe")
        np.add(p.indices, np.int32(rows[i]), out=indices[nnz[i]:nnz[i + 1]], dtype=np.int32, casting="unsafe")
        data[nnz[i]:nnz[i + 1]] = p.data
    out = sp.csr_matrix((data, indices, indptr), shape=(int(rows[-1]), int(rows[-1])))
    out.has_sorted_indices = True
    return out


class KPMBatch:
    """A ragged batch of independent models run together: every Chebyshev step of
    every model is one kernel launch over the block-diagonal matrix."""

    def __init__(self, models, energy_range=None, kernel=None, **kwargs):
        self.models = list(models)
        if not self.models:
            raise ValueError("empty model batch")
        self.kernel = kernel if kernel is not None else jackson_kernel()
        hs = [sp.csr_matrix(m.hamiltonian) for m in self.models]
        h = block_diagonal(hs)
        self.offsets = np.concatenate([[0], np.cumsum([x.shape[0] for x in hs])]).astype(np.int64)
        args = dict(energy_range=tuple(energy_range or (0, 0)), kernel=self.kernel.name,
                    kernel_param=self.kernel.param)
        args.update({k: v for k, v in kwargs.items() if k in ("matrix_format", "optimal_size", "interleaved",
                                                              "lanczos_precision", "precision", "batch_width",
                                                              "tile_rows", "fuse_steps", "staging")})
        self.engine = _binding.Engine(h, args, system_offsets=self.offsets)

    def scaling_factors(self):
        return [self.engine.scaling_factors(s) for s in range(len(self.models))]

    def calc_dos(self, energy, broadening, num_random=1):
        """DOS of every model (``KPM::calc_dos`` per model) as a list of :class:`Series`."""
        out = self.engine.calc_dos(energy, broadening, num_random)
        return [Series(energy, d, labels=dict(variable="E (eV)", data="DOS")) for d in out]

    def moments(self, num_moments, starters, average=False):
        """Diagonal moments of every model for supplied starters ``[model][vector][site]``."""
        return self.engine.moments_diag(num_moments, starters, average=average)

    def calc_ldos(self, energy, broadening, position=None, sublattice="", sites=None):
        """LDOS of every model (``KPM::calc_ldos`` per model, single-orbital models) at the site
        nearest to ``position`` (one position for all models, or one per model), or at the
        Hamiltonian rows ``sites``; all models in one recursion. A list of :class:`Series`."""
        if sites is None:
            pos = list(position) if (position is not None and np.ndim(position) == 2) else [position] * len(self.models)
            if len(pos) != len(self.models):
                raise ValueError("give one position, or one per model")
            sites = []
            for m, p in zip(self.models, pos):
                idx = np.atleast_1d(m.system.to_hamiltonian_indices(m.system.find_nearest(p, sublattice)))
                if idx.size != 1:
                    raise ValueError("batched LDOS needs single-orbital models")
                sites.append(int(idx[0]))
        out = self.engine.calc_ldos_batch(sites, energy, broadening)
        return [Series(energy, d, labels=dict(variable="E (eV)", data="LDOS", columns="orbitals")) for d in out]

    def close(self):
        self.engine.close()


def kpm_batch(models, energy_range=None, kernel="default", **kwargs):
    """Batch several models of uneven size into one GPU recursion (see :class:`KPMBatch`)."""
    return KPMBatch(models, energy_range, None if kernel == "default" else kernel, **kwargs)
