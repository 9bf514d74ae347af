"""ctypes front end of the KPM oracle (oracle/kpm_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the CPU restatement of pybinding's KPM that checks
the GPU engine. Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline legs import this module; the product (pybinding_gb300) never does.

The library is compiled from source on first use (``build()``), into
``oracle/_build/`` on whichever machine runs it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libkpm_oracle.so")
SRC = os.path.join(HERE, "kpm_oracle.cpp")

_lock = threading.Lock()
_lib = None

DTYPE_CODE = {np.dtype(np.float32): 0, np.dtype(np.float64): 1,
              np.dtype(np.complex64): 2, np.dtype(np.complex128): 3}
KERNELS = {"jackson": 0, "lorentz": 1, "dirichlet": 2}


# The timed CPU baseline is the same source built for speed on the host that runs it: FMA
# contraction on, complex products without the C99 NaN/Inf recovery (the reference's SIMD
# complex arithmetic has none), and on aarch64 (the GPU host's Grace CPU) tuned with
# -mcpu=native. Its results are never compared bit for bit; parity uses LIB_PATH.
FAST_LIB_PATH = os.path.join(BUILD_DIR, "libkpm_cpu_timed.so")


def _fast_flags():
    import platform
    flags = ["-O3", "-ffp-contract=fast", "-fcx-limited-range"]
    if platform.machine() in ("aarch64", "arm64"):
        flags.append("-mcpu=native")
    return flags


def _compile(out, flags):
    tmp = out + ".%d.tmp" % os.getpid()
    cmd = ["g++", "-std=c++17"] + flags + ["-fPIC", "-shared", "-pthread", "-Wno-psabi", SRC, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, out)


def _fresh(path):
    return os.path.exists(path) and os.path.getmtime(path) >= os.path.getmtime(SRC)


def build(force=False):
    """Compile the oracle (g++, C++17, -O3; FMA contraction off for cross-host repeatability)
    and the timed CPU baseline library (see FAST_LIB_PATH)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    jobs = []
    if force or not _fresh(LIB_PATH):
        jobs.append((LIB_PATH, ["-O3", "-ffp-contract=off"]))
    if force or not _fresh(FAST_LIB_PATH):
        jobs.append((FAST_LIB_PATH, _fast_flags()))
    if len(jobs) == 2:
        t = threading.Thread(target=_compile, args=jobs[1])
        t.start()
        _compile(*jobs[0])
        t.join()
        if not _fresh(FAST_LIB_PATH):
            raise RuntimeError("building %s failed" % FAST_LIB_PATH)
    elif jobs:
        _compile(*jobs[0])
    return LIB_PATH


class Config(C.Structure):
    _fields_ = [("min_energy", C.c_double), ("max_energy", C.c_double), ("kernel", C.c_int32),
                ("lam", C.c_double), ("optimal_size", C.c_int32), ("interleaved", C.c_int32),
                ("ell", C.c_int32), ("lanczos_precision", C.c_double)]


def make_config(energy_range=(0.0, 0.0), kernel="jackson", lam=4.0, matrix_format="ELL",
                optimal_size=True, interleaved=True, lanczos_precision=0.002):
    return Config(float(energy_range[0]), float(energy_range[1]), KERNELS[kernel], float(lam),
                  int(optimal_size), int(interleaved), int(matrix_format == "ELL"), float(lanczos_precision))


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = C.CDLL(LIB_PATH)
            _lib.orc_last_error.restype = C.c_char_p
            for name in ("orc_round_num_moments", "orc_required_num_moments", "orc_slicemap_index"):
                getattr(_lib, name).restype = C.c_int64
            _lib.orc_required_num_moments.argtypes = [C.c_int32, C.c_double, C.c_double]
            _lib.orc_round_num_moments.argtypes = [C.c_int64]
            _lib.orc_slicemap_index.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64]
            _lib.orc_scale.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_void_p]
            _lib.orc_damping.argtypes = [C.c_int32, C.c_double, C.c_int64, C.c_void_p]
        return _lib


_fast = None


def timed_lib():
    """The timed CPU baseline build of the same source (FAST_LIB_PATH)."""
    global _fast
    with _lock:
        if _fast is None:
            build()
            _fast = C.CDLL(FAST_LIB_PATH)
            _fast.orc_last_error.restype = C.c_char_p
        return _fast


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _check(rc, from_lib=None):
    if rc != 0:
        msg = (from_lib or lib()).orc_last_error().decode()
        raise (ValueError if rc == 2 else RuntimeError)(msg)


def _csr(h):
    h = sp.csr_matrix(h)
    h.sort_indices()
    ip = np.ascontiguousarray(h.indptr, dtype=np.int32)
    ix = np.ascontiguousarray(h.indices, dtype=np.int32)
    v = np.ascontiguousarray(h.data)
    return h.shape[0], ip, ix, v, DTYPE_CODE[v.dtype]


def _i64(x):
    return C.c_int64(int(x))


# ----------------------------------------------------------------- small helpers

def scale(emin, emax):
    a, b = C.c_double(), C.c_double()
    lib().orc_scale(emin, emax, C.byref(a), C.byref(b))
    return a.value, b.value


def round_num_moments(n):
    return int(lib().orc_round_num_moments(int(n)))


def required_num_moments(kernel, lam, scaled_broadening):
    return int(lib().orc_required_num_moments(KERNELS[kernel], lam, scaled_broadening))


def damping(kernel, lam, n):
    out = np.empty(n, np.float64)
    lib().orc_damping(KERNELS[kernel], lam, int(n), _p(out))
    return out


def slicemap_index(slices, src_off, dest_off, n, M):
    s = np.ascontiguousarray(slices, np.int32)
    return int(lib().orc_slicemap_index(_p(s), s.size, src_off, dest_off, n, M))


# ----------------------------------------------------------------- building blocks

def lanczos(h, precision_percent=0.002):
    """Extreme eigenvalues by Lanczos in H's scalar type (compute/lanczos.hpp:101-154)."""
    n, ip, ix, v, dt = _csr(h)
    mn, mx, loops = C.c_double(), C.c_double(), C.c_int32()
    _check(lib().orc_lanczos(dt, _i64(n), _p(ip), _p(ix), _p(v), C.c_double(float(np.float32(precision_percent))),
                             C.byref(mn), C.byref(mx), C.byref(loops)))
    return mn.value, mx.value, loops.value


def optimize(h, src, dest, a, b, reorder=True):
    """create_reordered / create_scaled (kpm/OptimizedHamiltonian.cpp:55-152)."""
    n, ip, ix, v, dt = _csr(h)
    src = np.ascontiguousarray(np.atleast_1d(src), np.int32)
    dest = np.ascontiguousarray(np.atleast_1d(dest), np.int32)
    cap = ip[-1] + n
    oip = np.empty(n + 1, np.int32)
    oix = np.empty(cap, np.int32)
    ov = np.empty(cap, v.dtype)
    omap = np.empty(n, np.int32)
    osl = np.empty(n + 1, np.int32)
    osrc = np.empty(src.size, np.int32)
    odest = np.empty(dest.size, np.int32)
    nnz, nsl, so, do = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
    _check(lib().orc_optimize(dt, _i64(n), _p(ip), _p(ix), _p(v), _p(src), _i64(src.size), _p(dest),
                              _i64(dest.size), C.c_double(a), C.c_double(b), C.c_int32(int(reorder)),
                              _p(oip), _p(oix), _p(ov), C.byref(nnz), _p(omap), _p(osl), C.byref(nsl),
                              _p(osrc), _p(odest), C.byref(so), C.byref(do)))
    h2 = sp.csr_matrix((ov[:nnz.value].copy(), oix[:nnz.value].copy(), oip.copy()), shape=(n, n))
    return dict(h2=h2, reorder_map=omap, slices=osl[:nsl.value].copy(), src=osrc, dest=odest,
                src_offset=so.value, dest_offset=do.value)


def random_starters(n, count, dtype, op=None):
    """``count`` reference random starters in draw order, original site order (Starter.cpp:48-84)."""
    dtype = np.dtype(dtype)
    out = np.empty((count, n), dtype)
    if op is not None:
        on, oip, oix, ov, _ = _csr(sp.csr_matrix(op).astype(dtype))
    else:
        on, oip, oix, ov = 0, None, None, None
    _check(lib().orc_random_starters(DTYPE_CODE[dtype], _i64(n), _i64(count), _i64(on), _p(oip), _p(oix), _p(ov),
                                     _p(out)))
    return out


def reorder_vector(v, reorder_map):
    out = np.empty_like(v)
    out[..., reorder_map] = v
    return out


def moments_diag(h2, r0, M, slices=None, src_offset=0, dest_offset=0, ell=True, optimal_size=False,
                 interleaved=True):
    """Diagonal moments for starters ``r0`` (k, n) on an optimized matrix -> (k, M)."""
    n, ip, ix, v, dt = _csr(h2)
    r0 = np.ascontiguousarray(np.atleast_2d(r0), v.dtype)
    sl = np.ascontiguousarray(slices if slices is not None else [n], np.int32)
    out = np.empty((r0.shape[0], M), v.dtype)
    _check(lib().orc_moments_diag(dt, _i64(n), _p(ip), _p(ix), _p(v), _p(sl), _i64(sl.size), _i64(src_offset),
                                  _i64(dest_offset), C.c_int32(int(ell)), C.c_int32(int(optimal_size)),
                                  C.c_int32(int(interleaved)), _p(r0), _i64(r0.shape[0]), _i64(M), _p(out)))
    return out


def moments_offdiag(h2, r0, beta, M, ell=True, interleaved=False):
    n, ip, ix, v, dt = _csr(h2)
    r0 = np.ascontiguousarray(r0, v.dtype)
    beta = np.ascontiguousarray(beta, v.dtype)
    out = np.empty(M, v.dtype)
    _check(lib().orc_moments_offdiag(dt, _i64(n), _p(ip), _p(ix), _p(v), C.c_int32(int(ell)),
                                     C.c_int32(int(interleaved)), _p(r0), _p(beta), _i64(M), _p(out)))
    return out


def dense_vectors(h2, r0, M):
    n, ip, ix, v, dt = _csr(h2)
    r0 = np.ascontiguousarray(r0, v.dtype)
    out = np.empty((M, n), v.dtype)
    _check(lib().orc_dense_vectors(dt, _i64(n), _p(ip), _p(ix), _p(v), _p(r0), _i64(M), _p(out)))
    return out


def velocity(h, alpha):
    n, ip, ix, v, dt = _csr(h)
    alpha = np.ascontiguousarray(alpha, np.float32)
    out = np.empty_like(v)
    _check(lib().orc_velocity(dt, _i64(n), _p(ip), _p(ix), _p(v), _p(alpha), _p(out)))
    return sp.csr_matrix((out, ix, ip), shape=(n, n))


def spectral_density(moments, energy, a, b, dtype):
    m = np.ascontiguousarray(np.atleast_2d(np.asarray(moments).T).T, np.complex128)  # (M, cols)
    M, cols = m.shape
    m = np.ascontiguousarray(m.T)
    e = np.ascontiguousarray(energy, np.float64)
    out = np.empty((cols, e.size), np.float64)
    _check(lib().orc_spectral_density(DTYPE_CODE[np.dtype(dtype)], _p(m), _i64(M), _i64(cols), _p(e), _i64(e.size),
                                      C.c_double(a), C.c_double(b), _p(out)))
    return out.T


def greens_function(moments, energy, a, b, dtype):
    m = np.ascontiguousarray(moments, np.complex128)
    e = np.ascontiguousarray(energy, np.float64)
    out = np.empty(e.size, np.complex128)
    _check(lib().orc_greens_function(DTYPE_CODE[np.dtype(dtype)], _p(m), _i64(m.size), _p(e), _i64(e.size),
                                     C.c_double(a), C.c_double(b), _p(out)))
    return out


def kubo_bastin(mu, chem, samples, temperature, a, b, dtype):
    mu = np.asfortranarray(mu, np.complex128)
    M = mu.shape[0]
    ch = np.ascontiguousarray(chem, np.float64)
    s = np.ascontiguousarray(samples, np.float64)
    out = np.empty(ch.size, np.complex128)
    _check(lib().orc_kubo_bastin(DTYPE_CODE[np.dtype(dtype)], mu.ctypes.data_as(C.c_void_p), _i64(M), _p(ch),
                                 _i64(ch.size), _p(s), _i64(s.size), C.c_double(temperature), C.c_double(a),
                                 C.c_double(b), _p(out)))
    return out


# ----------------------------------------------------------------- Core-level flows

def core_dos(h, energy, broadening, num_random=1, **cfg):
    n, ip, ix, v, dt = _csr(h)
    e = np.ascontiguousarray(energy, np.float64)
    out = np.empty(e.size, np.float64)
    ab = np.empty(4, np.float64)
    c = make_config(**cfg)
    _check(lib().orc_core_dos(dt, _i64(n), _p(ip), _p(ix), _p(v), C.byref(c), _p(e), _i64(e.size),
                              C.c_double(broadening), _i64(num_random), _p(out), _p(ab)))
    return out, ab


def core_ldos(h, idx, energy, broadening, **cfg):
    n, ip, ix, v, dt = _csr(h)
    idx = np.ascontiguousarray(np.atleast_1d(idx), np.int32)
    e = np.ascontiguousarray(energy, np.float64)
    out = np.empty((idx.size, e.size), np.float64)
    c = make_config(**cfg)
    _check(lib().orc_core_ldos(dt, _i64(n), _p(ip), _p(ix), _p(v), C.byref(c), _p(idx), _i64(idx.size), _p(e),
                               _i64(e.size), C.c_double(broadening), _p(out)))
    return out.T


def core_greens(h, row, cols, energy, broadening, **cfg):
    n, ip, ix, v, dt = _csr(h)
    cols = np.ascontiguousarray(np.atleast_1d(cols), np.int32)
    e = np.ascontiguousarray(energy, np.float64)
    out = np.empty((cols.size, e.size), np.complex128)
    c = make_config(**cfg)
    _check(lib().orc_core_greens(dt, _i64(n), _p(ip), _p(ix), _p(v), C.byref(c), C.c_int32(int(row)), _p(cols),
                                 _i64(cols.size), _p(e), _i64(e.size), C.c_double(broadening), _p(out)))
    return out


def core_moments(h, num_moments, alpha, beta=None, op=None, **cfg):
    n, ip, ix, v, dt = _csr(h)
    a = np.ascontiguousarray(alpha, np.complex128)
    b = np.ascontiguousarray(beta, np.complex128) if beta is not None and len(beta) else None
    if op is not None and op.shape[0] != 0:
        on, oip, oix, ov, _ = _csr(sp.csr_matrix(op).astype(np.complex128))
    else:
        on, oip, oix, ov = 0, None, None, None
    out = np.empty(num_moments, np.complex128)
    c = make_config(**cfg)
    _check(lib().orc_core_moments(dt, _i64(n), _p(ip), _p(ix), _p(v), C.byref(c), _i64(num_moments), _p(a), _p(b),
                                  _i64(on), _p(oip), _p(oix), _p(ov), _p(out)))
    return out


def core_conductivity(h, left, right, chem, broadening, temperature, num_random=1, num_points=1000, **cfg):
    n, ip, ix, v, dt = _csr(h)
    l_ = np.ascontiguousarray(left, np.float32)
    r_ = np.ascontiguousarray(right, np.float32)
    ch = np.ascontiguousarray(chem, np.float64)
    out = np.empty(ch.size, np.complex128)
    c = make_config(**cfg)
    _check(lib().orc_core_conductivity(dt, _i64(n), _p(ip), _p(ix), _p(v), C.byref(c), _p(l_), _p(r_), _p(ch),
                                       _i64(ch.size), C.c_double(broadening), C.c_double(temperature),
                                       _i64(num_random), _i64(num_points), _p(out)))
    return out


# ----------------------------------------------------------------- timed CPU baseline

def bench_diag(h2, slices, r0, M, k, threads):
    """Time the multithreaded restatement of DefaultCompute's DOS batches.

    ``r0`` is (R, n) in the optimized matrix's order. Returns (moments (R, M), seconds).
    """
    n, ip, ix, v, dt = _csr(h2)
    r0 = np.ascontiguousarray(r0, v.dtype)
    sl = np.ascontiguousarray(slices, np.int32)
    R = r0.shape[0]
    out = np.empty((R, M), v.dtype)
    sec = C.c_double()
    _check(timed_lib().orc_bench_diag(dt, _i64(n), _p(ip), _p(ix), _p(v), _p(sl), _i64(sl.size), _p(r0), _i64(R),
                                      _i64(M), _i64(k), C.c_int32(int(threads)), _p(out), C.byref(sec)), timed_lib())
    return out, sec.value


def bench_diag_multi(systems, M, k, threads):
    """The timed baseline over several systems at once, every (system, batch) pair on one pool.

    ``systems``: list of (h2, slices, r0) with r0 (R, n) in h2's order, the same R and scalar
    type for all. Returns (moments (nsys, R, M), seconds).
    """
    ns = len(systems)
    keep, n, ip, ix, v, sl, nsl, r0 = [], [], [], [], [], [], [], []
    dt = None
    R = None
    for h2, slices, r in systems:
        nn, a, b, c, d = _csr(h2)
        dt = d if dt is None else dt
        if d != dt:
            raise ValueError("all systems must have one scalar type")
        r = np.ascontiguousarray(r, c.dtype)
        R = r.shape[0] if R is None else R
        if r.shape != (R, nn):
            raise ValueError("starters must be (R, n) with one R for all systems")
        s_ = np.ascontiguousarray(slices, np.int32)
        keep += [a, b, c, r, s_]
        n.append(nn)
        ip.append(a.ctypes.data); ix.append(b.ctypes.data); v.append(c.ctypes.data)
        sl.append(s_.ctypes.data); nsl.append(s_.size); r0.append(r.ctypes.data)
    ptrs = lambda xs: (C.c_void_p * ns)(*xs)
    n_ = np.asarray(n, np.int64)
    nsl_ = np.asarray(nsl, np.int64)
    out = np.empty((ns, R, M), keep[2].dtype)
    sec = C.c_double()
    _check(timed_lib().orc_bench_diag_multi(dt, C.c_int32(ns), _p(n_), ptrs(ip), ptrs(ix), ptrs(v), ptrs(sl),
                                            _p(nsl_), ptrs(r0), _i64(R), _i64(M), _i64(k), C.c_int32(int(threads)),
                                            _p(out), C.byref(sec)), timed_lib())
    return out, sec.value
