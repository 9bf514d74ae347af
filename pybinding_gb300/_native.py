"""ctypes binding of the engine's C ABI (include/kpm_gb300.h, include/kpm_lattice.h).

The shared library is built in-tree (``pybinding_gb300/_build/libkpm_gb300.so``)
by ``pybinding_gb300.build``. Loading fails loudly when it is missing: there is
no CPU fallback for any computation in this package.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

_lock = threading.Lock()
_lib = None

KPM_OK, KPM_ERR_RUNTIME, KPM_ERR_VALUE, KPM_ERR_CUDA, KPM_ERR_TIMEOUT = 0, 1, 2, 3, 4
SCALAR_CODE = {np.dtype(np.float32): 0, np.dtype(np.float64): 1,
               np.dtype(np.complex64): 2, np.dtype(np.complex128): 3}
KERNEL_CODE = {"jackson": 0, "lorentz": 1, "dirichlet": 2}
PRECISION_CODE = {"auto": 0, "fp64": 1, "fp32": 2, "fp32x": 3, "fp32p": 4}
STAGING_CODE = {"auto": 0, "registers": 1, "prefetch": 2}


PROGRESS_FN = C.CFUNCTYPE(None, C.c_int64, C.c_int64, C.c_void_p)


class Config(C.Structure):
    """kpm_config (include/kpm_gb300.h)"""
    _fields_ = [("min_energy", C.c_double), ("max_energy", C.c_double), ("kernel", C.c_int32),
                ("kernel_param", C.c_double), ("matrix_format", C.c_int32), ("optimal_size", C.c_int32),
                ("interleaved", C.c_int32), ("lanczos_precision", C.c_double), ("precision", C.c_int32),
                ("batch_width", C.c_int32), ("tile_rows", C.c_int32), ("fuse_steps", C.c_int32),
                ("staging", C.c_int32), ("num_threads", C.c_int32)]


class Stats(C.Structure):
    """kpm_stats (include/kpm_gb300.h)"""
    _fields_ = [("num_moments", C.c_int64), ("uses_full_system", C.c_int32), ("nnz", C.c_int64),
                ("opt_nnz", C.c_int64), ("vec", C.c_int64), ("opt_vec", C.c_int64), ("multiplier", C.c_double),
                ("matrix_memory", C.c_int64), ("vector_memory", C.c_int64), ("hamiltonian_time", C.c_double),
                ("moments_time", C.c_double), ("bounds_time", C.c_double), ("lanczos_loops", C.c_int32),
                ("eps", C.c_double), ("steps_per_launch", C.c_int32), ("gemm_time", C.c_double),
                ("elems_per_lane", C.c_int32), ("lanes_per_row", C.c_int32), ("staged_rows", C.c_int32),
                ("tile_rows", C.c_int32), ("unroll", C.c_int32), ("upload_time", C.c_double),
                ("call_time", C.c_double), ("gather_rows", C.c_int32), ("prefetch", C.c_int32)]


class Honeycomb(C.Structure):
    """kpm_honeycomb (include/kpm_lattice.h)"""
    _fields_ = [("s0", C.c_int32), ("s1", C.c_int32), ("origin", C.c_float * 3), ("a1", C.c_float * 3),
                ("a2", C.c_float * 3), ("sub", (C.c_float * 3) * 2), ("hop", (C.c_int32 * 2) * 3),
                ("min_neighbors", C.c_int32)]


# every exported symbol of include/kpm_gb300.h and include/kpm_lattice.h with (restype, argtypes)
_P, _I32, _I64, _D = C.c_void_p, C.c_int32, C.c_int64, C.c_double
SIGNATURES = {
    "kpm_last_error": (C.c_char_p, []),
    "kpm_config_default": (None, [_P]),
    "kpm_create": (_I32, [_I32, _I64, _P, _P, _P, _I32, _P, _P, _P]),
    "kpm_destroy": (_I32, [_P]),
    "kpm_create_batch": (_I32, [_P, _I32, _P, _P]),
    "kpm_set_hamiltonian": (_I32, [_P, _I32, _I64, _P, _P, _P, _I32, _P]),
    "kpm_energy_bounds": (_I32, [_P, _I32, _P, _P, _P]),
    "kpm_scaling_factors": (_I32, [_P, _I32, _P, _P]),
    "kpm_moments_diag": (_I32, [_P, _I64, _I64, _P, _I32, _I32, _P, _P]),
    "kpm_calc_dos": (_I32, [_P, _P, _I64, _D, _I64, _P]),
    "kpm_calc_ldos": (_I32, [_P, _P, _I64, _P, _I64, _D, _P]),
    "kpm_calc_ldos_batch": (_I32, [_P, _P, _P, _I64, _D, _P]),
    "kpm_calc_greens": (_I32, [_P, _I64, _P, _I64, _P, _I64, _D, _P]),
    "kpm_moments": (_I32, [_P, _I64, _P, _I64, _P, _I64, _I64, _P, _P, _P, _P]),
    "kpm_calc_conductivity": (_I32, [_P, _P, _P, _P, _I64, _D, _D, _I64, _I64, _I32, _P]),
    "kpm_adjoint_diag": (_I32, [_P, _I64, _I64, _P, _P, _I64, _P, _P, _P]),
    "kpm_adjoint_conductivity": (_I32, [_P, _P, _P, _I64, _I64, _P, _P, _P, _P, _P]),
    "kpm_conductivity_moments": (_I32, [_P, _P, _P, _I64, _I64, _I32, _P]),
    "kpm_kubo_bastin": (_I32, [_P, _P, _I64, _P, _I64, _D, _I64, _P]),
    "kpm_get_stats": (_I32, [_P, _P]),
    "kpm_report": (_I32, [_P, _I32, _P, _I64]),
    "kpm_optimized_hamiltonian": (_I32, [_P, _P, _I64, _P, _I64, _I32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "kpm_get_stream": (_I32, [_P, _P]),
    "kpm_set_progress_callback": (_I32, [_P, PROGRESS_FN, _P]),
    "kpm_moments_diag_noalloc": (_I32, [_I32, _I64, _I32, _P, _P, _I64, _P, _P, _I64, _P, _P]),
    "kpm_damping_coefficients": (_I32, [_I32, _D, _I64, _P]),
    "kpm_required_num_moments": (_I64, [_I32, _D, _D]),
    # include/kpm_lattice.h
    "kpm_lattice_honeycomb": (_I32, [_P, _P, _I32, _P]),
    "kpm_lattice_cubic": (_I32, [_I32, _P]),
    "kpm_lattice_sizes": (_I32, [_P, _P, _P, _P, _P]),
    "kpm_lattice_sites": (_I32, [_P, _P, _P, _P]),
    "kpm_lattice_hoppings": (_I32, [_P, _P, _P]),
    "kpm_lattice_csr": (_I32, [_P, _I32, _P, _P, _P, _P, _P, _P, _I64, _P]),
    "kpm_lattice_times": (_I32, [_P, _P, _P, _P]),
    "kpm_lattice_destroy": (_I32, [_P]),
}


def library_path():
    return _build.LIB


def lib():
    """Load (building first if needed) the engine library; raise if it cannot be loaded."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not os.path.exists(path) or _build._stale():
                try:
                    _build.build()
                except Exception as e:  # no toolchain: the product cannot run
                    raise ImportError("pybinding_gb300: the CUDA engine library is missing and could not be "
                                      "built (%s). There is no CPU fallback." % e) from e
            handle = C.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
        return _lib


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def check(rc):
    if rc != KPM_OK:
        msg = lib().kpm_last_error().decode()
        if rc == KPM_ERR_VALUE:
            raise ValueError(msg)
        raise RuntimeError(msg)


def make_config(energy_range=(0.0, 0.0), kernel="jackson", kernel_param=4.0, matrix_format="ELL",
                optimal_size=True, interleaved=True, lanczos_precision=0.002, precision="auto", batch_width=0,
                tile_rows=0, fuse_steps=0, staging="auto", num_threads=0):
    c = Config()
    lib().kpm_config_default(C.byref(c))
    c.min_energy, c.max_energy = float(energy_range[0]), float(energy_range[1])
    c.kernel = KERNEL_CODE[kernel]
    c.kernel_param = float(kernel_param)
    c.matrix_format = 1 if matrix_format == "ELL" else 0
    c.optimal_size = int(bool(optimal_size))
    c.interleaved = int(bool(interleaved))
    c.lanczos_precision = float(lanczos_precision)
    c.precision = PRECISION_CODE[precision]
    c.batch_width = int(batch_width)
    c.tile_rows = int(tile_rows)
    c.fuse_steps = int(fuse_steps)
    c.staging = STAGING_CODE[staging]
    c.num_threads = 0 if num_threads in (None, "auto") else int(num_threads)
    return c


class Engine:
    """Owner of one native engine handle (one device stream, device buffers)."""

    def __init__(self, hamiltonian, config, system_offsets=None):
        self._h = None
        self.config = config
        self._set(hamiltonian, system_offsets, create=True)

    @staticmethod
    def _csr_arrays(h):
        import scipy.sparse as sp
        h = sp.csr_matrix(h)
        if not h.has_sorted_indices:
            h = h.copy()
            h.sort_indices()
        dtype = np.dtype(h.dtype)
        if dtype not in SCALAR_CODE:
            raise TypeError("unsupported Hamiltonian dtype %s" % dtype)
        ip = np.ascontiguousarray(h.indptr, np.int32)
        ix = np.ascontiguousarray(h.indices, np.int32)
        v = np.ascontiguousarray(h.data)
        return h.shape[0], ip, ix, v, SCALAR_CODE[dtype]

    def _set(self, h, offsets, create=False):
        n, ip, ix, v, st = self._csr_arrays(h)
        off = None if offsets is None else np.ascontiguousarray(offsets, np.int64)
        ns = 1 if off is None else off.size - 1
        self.rows, self.num_systems, self.dtype = n, ns, np.dtype(v.dtype)
        self._nnz = int(ip[-1])
        self.system_offsets = np.array([0, n], np.int64) if off is None else off
        if create:
            handle = C.c_void_p()
            check(lib().kpm_create(st, n, ptr(ip), ptr(ix), ptr(v), ns, ptr(off), C.byref(self.config),
                                   C.byref(handle)))
            self._h = handle
        else:
            check(lib().kpm_set_hamiltonian(self._h, st, n, ptr(ip), ptr(ix), ptr(v), ns, ptr(off)))

    def set_hamiltonian(self, h, system_offsets=None):
        self._set(h, system_offsets)

    @classmethod
    def from_engines(cls, engines, config):
        """A ragged-batch engine whose system i is the Hamiltonian of ``engines[i]`` (single-system
        engines of one scalar type), made without copying the matrices through Python
        (``kpm_create_batch``)."""
        engines = list(engines)
        arr = (C.c_void_p * len(engines))(*[e._h for e in engines])
        handle = C.c_void_p()
        check(lib().kpm_create_batch(arr, len(engines), C.byref(config), C.byref(handle)))
        self = cls.__new__(cls)
        self._h = handle
        self.config = config
        sizes = [e.rows for e in engines]
        self.rows, self.num_systems, self.dtype = int(sum(sizes)), len(engines), engines[0].dtype
        self._nnz = int(sum(e._nnz for e in engines))
        self.system_offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        return self

    def close(self):
        if self._h is not None and _lib is not None:
            lib().kpm_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # ------------------------------------------------------------------ calls
    def energy_bounds(self, system=0):
        mn, mx, loops = C.c_double(), C.c_double(), C.c_int32()
        check(lib().kpm_energy_bounds(self._h, system, C.byref(mn), C.byref(mx), C.byref(loops)))
        return mn.value, mx.value, loops.value

    def scaling_factors(self, system=0):
        a, b = C.c_double(), C.c_double()
        check(lib().kpm_scaling_factors(self._h, system, C.byref(a), C.byref(b)))
        return a.value, b.value

    def moments_diag(self, num_moments, starters, average=False, on_device_ptr=None, num_vectors=None):
        """Diagonal moments for supplied starters ``[system][vector][site]``.

        ``starters`` is a host array (converted to the Hamiltonian's dtype), or
        ``on_device_ptr`` is the address of a device buffer that already holds
        ``num_vectors * rows`` elements of the Hamiltonian's dtype in that layout.
        """
        nout = C.c_int64()
        rounded = round_num_moments(num_moments)
        if on_device_ptr is not None:
            if num_vectors is None or int(num_vectors) < 1:
                raise ValueError("num_vectors is required with a device pointer")
            nvec = int(num_vectors)
            src, dev, keep = C.c_void_p(int(on_device_ptr)), 1, None
        else:
            keep = np.ascontiguousarray(starters, dtype=self.dtype)
            if keep.size == 0 or keep.size % self.rows:
                raise ValueError("starters must hold num_vectors * %d elements" % self.rows)
            nvec = keep.size // self.rows
            src, dev = ptr(keep), 0
        cols = self.num_systems if average else self.num_systems * nvec
        out = np.empty((cols, rounded), np.complex128)
        check(lib().kpm_moments_diag(self._h, num_moments, nvec, src, dev, int(bool(average)), ptr(out),
                                     C.byref(nout)))
        del keep
        shape = (self.num_systems, rounded) if average else (self.num_systems, nvec, rounded)
        return out.reshape(shape)

    def calc_dos(self, energy, broadening, num_random):
        e = np.ascontiguousarray(energy, np.float64)
        out = np.empty((self.num_systems, e.size), np.float64)
        check(lib().kpm_calc_dos(self._h, ptr(e), e.size, float(broadening), int(num_random), ptr(out)))
        return out

    def calc_ldos(self, indices, energy, broadening):
        idx = np.ascontiguousarray(np.atleast_1d(indices), np.int64)
        e = np.ascontiguousarray(energy, np.float64)
        out = np.empty((idx.size, e.size), np.float64)
        check(lib().kpm_calc_ldos(self._h, ptr(idx), idx.size, ptr(e), e.size, float(broadening), ptr(out)))
        return out.T  # (energy, indices)

    def calc_ldos_batch(self, sites, energy, broadening):
        """LDOS of every system at one local site each: [num_systems][num_energy]."""
        sites = np.ascontiguousarray(sites, dtype=np.int64)
        if sites.size != self.num_systems:
            raise ValueError("one LDOS site per system (%d)" % self.num_systems)
        e = np.ascontiguousarray(energy, dtype=np.float64)
        out = np.empty((self.num_systems, e.size))
        check(lib().kpm_calc_ldos_batch(self._h, ptr(sites), ptr(e), e.size, float(broadening), ptr(out)))
        return out

    def calc_greens(self, row, cols, energy, broadening):
        c = np.ascontiguousarray(np.atleast_1d(cols), np.int64)
        e = np.ascontiguousarray(energy, np.float64)
        out = np.empty((c.size, e.size), np.complex128)
        check(lib().kpm_calc_greens(self._h, int(row), ptr(c), c.size, ptr(e), e.size, float(broadening), ptr(out)))
        return out

    def moments(self, num_moments, alpha, beta=None, op=None):
        a = np.ascontiguousarray(np.asarray(alpha).ravel(), np.complex128)
        b = None if beta is None or np.size(beta) == 0 else np.ascontiguousarray(np.asarray(beta).ravel(), np.complex128)
        if op is not None and op.shape[0] != 0:
            import scipy.sparse as sp
            o = sp.csr_matrix(op).astype(np.complex128)
            oip = np.ascontiguousarray(o.indptr, np.int32)
            oix = np.ascontiguousarray(o.indices, np.int32)
            ov = np.ascontiguousarray(o.data, np.complex128)
            orows = o.shape[0]
            if o.shape[0] != o.shape[1]:
                orows = -1
        else:
            oip = oix = ov = None
            orows = 0
        out = np.empty(int(num_moments), np.complex128)
        check(lib().kpm_moments(self._h, int(num_moments), ptr(a), a.size, ptr(b), 0 if b is None else b.size,
                                orows, ptr(oip), ptr(oix), ptr(ov), ptr(out)))
        return out

    def calc_conductivity(self, left, right, chemical_potential, broadening, temperature, num_random, num_points,
                          gemm_mode=0):
        l_ = np.ascontiguousarray(left, np.float32)
        r_ = np.ascontiguousarray(right, np.float32)
        mu = np.ascontiguousarray(np.atleast_1d(chemical_potential), np.float64)
        out = np.empty(mu.size, np.complex128)
        check(lib().kpm_calc_conductivity(self._h, ptr(l_), ptr(r_), ptr(mu), mu.size, float(broadening),
                                          float(temperature), int(num_random), int(num_points), int(gemm_mode),
                                          ptr(out)))
        return out

    def conductivity_moments(self, left, right, num_moments, num_random, gemm_mode=0):
        """Undamped Kubo-Bastin moments matrix (num_moments, num_moments) complex: mu[m, n]."""
        l_ = np.ascontiguousarray(left, np.float32)
        r_ = np.ascontiguousarray(right, np.float32)
        M = int(num_moments)
        out = np.empty((M, M), np.complex128)  # row n = column n of mu
        check(lib().kpm_conductivity_moments(self._h, ptr(l_), ptr(r_), M, int(num_random), int(gemm_mode), ptr(out)))
        return out.T.copy()

    def kubo_bastin(self, moments, chemical_potential, temperature, num_points):
        """Kubo-Bastin conductivity (complex) from a damped moments matrix mu[m, n]."""
        m = np.asarray(moments, np.complex128)
        M = m.shape[0]
        col_major = np.ascontiguousarray(m.T)  # column n contiguous
        mu = np.ascontiguousarray(np.atleast_1d(chemical_potential), np.float64)
        out = np.empty(mu.size, np.complex128)
        check(lib().kpm_kubo_bastin(self._h, ptr(col_major), M, ptr(mu), mu.size, float(temperature), int(num_points),
                                    ptr(out)))
        return out

    def adjoint_diag(self, num_moments, starters, dl_dmu, checkpoint=0):
        """Gradient of L = sum_n dl_dmu[n] mu_n (mu: averaged diagonal moments of ``starters``
        [vector][site]) with respect to the stored entries of H (CSR order) and the onsite
        energies; returns (grad_values, grad_onsite), both float64."""
        rounded = round_num_moments(num_moments)
        w = np.ascontiguousarray(dl_dmu, np.float64)
        if w.size != rounded:
            raise ValueError("dl_dmu must hold round_num_moments(num_moments) = %d entries" % rounded)
        keep = np.ascontiguousarray(starters, dtype=self.dtype)
        if keep.size == 0 or keep.size % self.rows:
            raise ValueError("starters must hold num_vectors * %d elements" % self.rows)
        nvec = keep.size // self.rows
        gv = np.empty(self._nnz, np.float64)
        go = np.empty(self.rows, np.float64)
        nout = C.c_int64()
        check(lib().kpm_adjoint_diag(self._h, num_moments, nvec, ptr(keep), ptr(w), int(checkpoint), ptr(gv), ptr(go),
                                     C.byref(nout)))
        return gv, go

    def set_progress_callback(self, callback):
        """``callback(delta, total)`` during calc_dos (kpm_set_progress_callback); None turns it off."""
        if callback is None:
            self._progress = None
            check(lib().kpm_set_progress_callback(self._h, None, None))
            return
        fn = PROGRESS_FN(lambda delta, total, user: callback(int(delta), int(total)))
        self._progress = fn  # kept alive as long as the engine may call it
        check(lib().kpm_set_progress_callback(self._h, fn, None))

    def adjoint_conductivity(self, left, right, num_moments, starters, dl_dmu=None):
        """Kubo-Bastin moments matrix mu[m, n] (undamped, real) of ``starters`` [vector][site]
        and, with ``dl_dmu`` (M, M), the gradient of sum(dl_dmu * mu) with respect to the stored
        entries of H and the onsite energies: (mu, grad_values, grad_onsite)."""
        l_ = np.ascontiguousarray(left, np.float32)
        r_ = np.ascontiguousarray(right, np.float32)
        keep = np.ascontiguousarray(starters, dtype=self.dtype)
        if keep.size == 0 or keep.size % self.rows:
            raise ValueError("starters must hold num_vectors * %d elements" % self.rows)
        M = int(num_moments)
        mu = np.empty((M, M), np.float64)
        gv = go = w = None
        if dl_dmu is not None:
            w = np.ascontiguousarray(dl_dmu, np.float64)
            if w.shape != (M, M):
                raise ValueError("dl_dmu must have shape (%d, %d)" % (M, M))
            gv = np.empty(self._nnz, np.float64)
            go = np.empty(self.rows, np.float64)
        check(lib().kpm_adjoint_conductivity(self._h, ptr(l_), ptr(r_), M, keep.size // self.rows, ptr(keep), ptr(w),
                                             ptr(mu), ptr(gv), ptr(go)))
        return mu, gv, go

    def stream(self):
        """The engine's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        p = C.c_void_p()
        check(lib().kpm_get_stream(self._h, C.byref(p)))
        return p.value or 0

    def stats(self):
        s = Stats()
        check(lib().kpm_get_stats(self._h, C.byref(s)))
        return s

    def report(self, shortform=False):
        buf = C.create_string_buffer(4096)
        check(lib().kpm_report(self._h, int(bool(shortform)), buf, 4096))
        return buf.value.decode()

    def optimized_hamiltonian(self, src, dest, reorder=True):
        import scipy.sparse as sp
        s = np.ascontiguousarray(np.atleast_1d(src), np.int32)
        d = np.ascontiguousarray(np.atleast_1d(dest), np.int32)
        n = self.rows
        cap = self._nnz_cap()
        oip = np.empty(n + 1, np.int32)
        oix = np.empty(cap, np.int32)
        ov = np.empty(cap, self.dtype)
        omap = np.empty(n, np.int32)
        osl = np.empty(n + 1, np.int32)
        osrc = np.empty(s.size, np.int32)
        odest = np.empty(d.size, np.int32)
        offs = np.empty(2, np.int64)
        nnz, nsl = C.c_int64(), C.c_int64()
        check(lib().kpm_optimized_hamiltonian(self._h, ptr(s), s.size, ptr(d), d.size, int(bool(reorder)), ptr(oip),
                                              ptr(oix), ptr(ov), C.byref(nnz), ptr(omap), ptr(osl), C.byref(nsl),
                                              ptr(osrc), ptr(odest), ptr(offs)))
        h2 = sp.csr_matrix((ov[:nnz.value].copy(), oix[:nnz.value].copy(), oip.copy()), shape=(n, n))
        return dict(h2=h2, reorder_map=omap, slices=osl[:nsl.value].copy(), src=osrc, dest=odest,
                    src_offset=int(offs[0]), dest_offset=int(offs[1]))

    def _nnz_cap(self):
        return self._nnz + self.rows


def round_num_moments(n):
    """kpm/Kernel.hpp:9-13: (n - 2) % 4 == 0, at least 2"""
    n = int(n)
    if n < 2:
        return 2
    return n + (4 - (n - 2) % 4) % 4


def damping_coefficients(kernel, param, num_moments):
    out = np.empty(int(num_moments), np.float64)
    check(lib().kpm_damping_coefficients(KERNEL_CODE[kernel], float(param), int(num_moments), ptr(out)))
    return out


def required_num_moments(kernel, param, scaled_broadening):
    return int(lib().kpm_required_num_moments(KERNEL_CODE[kernel], float(param), float(scaled_broadening)))


class LatticeBuild:
    """Device-side build of a honeycomb flake or a periodic cubic lattice (kpm_lattice.h).

    ``sites()``, ``hoppings()`` and ``csr()`` copy the results to host numpy arrays.
    """

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def honeycomb(cls, s0, s1, origin, a1, a2, sub, hop, vertices, min_neighbors):
        p = Honeycomb()
        p.s0, p.s1 = int(s0), int(s1)
        for c in range(3):
            p.origin[c], p.a1[c], p.a2[c] = float(origin[c]), float(a1[c]), float(a2[c])
            p.sub[0][c], p.sub[1][c] = float(sub[0][c]), float(sub[1][c])
        for k in range(3):
            p.hop[k][0], p.hop[k][1] = int(hop[k][0]), int(hop[k][1])
        p.min_neighbors = int(min_neighbors)
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 2)
        h = C.c_void_p()
        check(lib().kpm_lattice_honeycomb(C.byref(p), ptr(v), v.shape[0], C.byref(h)))
        return cls(h)

    @classmethod
    def cubic(cls, L):
        h = C.c_void_p()
        check(lib().kpm_lattice_cubic(int(L), C.byref(h)))
        return cls(h)

    def close(self):
        if self._h is not None and self._h.value:
            lib().kpm_lattice_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sizes(self):
        v = [C.c_int64() for _ in range(4)]
        check(lib().kpm_lattice_sizes(self._h, *[C.byref(x) for x in v]))
        return tuple(int(x.value) for x in v)

    def sites(self):
        n = self.sizes()[0]
        x, y, z = (np.empty(n, np.float32) for _ in range(3))
        check(lib().kpm_lattice_sites(self._h, ptr(x), ptr(y), ptr(z)))
        return x, y, z

    def hoppings(self):
        nh = self.sizes()[2]
        rows, cols = np.empty(nh, np.int32), np.empty(nh, np.int32)
        check(lib().kpm_lattice_hoppings(self._h, ptr(rows), ptr(cols)))
        return rows, cols

    def csr(self, dtype, hopping=None, hopping_values=None, onsite=None):
        """(indptr, indices, values) of the Hamiltonian; ``hopping`` is one value for every
        bond, ``hopping_values`` one per bond in ``hoppings()`` order."""
        dtype = np.dtype(dtype)
        n, _, nh, max_nnz = self.sizes()
        one = None if hopping is None else np.array([hopping], dtype=dtype)
        hv = None if hopping_values is None else np.ascontiguousarray(hopping_values, dtype=dtype)
        if hv is not None and hv.size != nh:
            raise ValueError("hopping_values must hold one value per hopping (%d)" % nh)
        ons = None if onsite is None else np.ascontiguousarray(onsite, dtype=dtype)
        if ons is not None and ons.size != n:
            raise ValueError("onsite must hold one value per site (%d)" % n)
        indptr = np.empty(n + 1, np.int32)
        indices = np.empty(max_nnz, np.int32)
        values = np.empty(max_nnz, dtype)
        nnz = C.c_int64()
        check(lib().kpm_lattice_csr(self._h, SCALAR_CODE[dtype], ptr(one), ptr(hv), ptr(ons), ptr(indptr),
                                    ptr(indices), ptr(values), max_nnz, C.byref(nnz)))
        k = int(nnz.value)
        return indptr, indices[:k].copy(), values[:k].copy()

    def times(self):
        """(device seconds of the site build, of the last CSR assembly, kernels launched)"""
        b, c, k = C.c_double(), C.c_double(), C.c_int64()
        check(lib().kpm_lattice_times(self._h, C.byref(b), C.byref(c), C.byref(k)))
        return b.value, c.value, int(k.value)
