"""The FP32 row-sum forms of the diagonal step, emulated operation by operation in NumPy (each
FP32 operation evaluated in FP64 and rounded to FP32; an FMA rounded once), on a small
disordered graphene flake: the FMA-compensated rows (fma_compensated_term) and the TwoSum rows
(two_sum_term) keep the recursion's moments several times closer to the FP64 recursion than
chained FMAs, which is why the FMA-compensated form is the automatic FP32 precision. CPU only."""
import numpy as np
import scipy.sparse as sp

from pybinding_gb300 import lattice as L


def _f32(v):
    return v.astype(np.float32).astype(np.float64)


def _ell(h2):
    h2 = sp.csr_matrix(h2)
    h2.sort_indices()
    n = h2.shape[0]
    w = int(np.diff(h2.indptr).max())
    col = np.repeat(np.arange(n)[:, None], w, axis=1)
    val = np.zeros((n, w))
    cnt = np.diff(h2.indptr)
    for j in range(w):
        m = cnt > j
        col[m, j] = h2.indices[h2.indptr[:-1][m] + j]
        val[m, j] = h2.data[h2.indptr[:-1][m] + j]
    return col, val


def _row_sums(col, val, hi, lo, x, mode):
    s = np.zeros_like(x)
    l = np.zeros_like(x)
    for j in range(col.shape[1]):
        h, hl, xj = hi[:, j:j + 1], lo[:, j:j + 1], x[col[:, j]]
        if mode == "fp64":
            s = s + val[:, j:j + 1] * xj
        elif mode == "fma":  # chained FMAs (the lo parts in their own chain)
            s = _f32(h * xj + s)
            l = _f32(hl * xj + l)
        elif mode == "fma_compensated":  # fma_compensated_term
            p = _f32(h * xj)
            s1 = _f32(s + p)
            c = _f32(h * xj + _f32(s - s1))
            l = _f32(hl * xj + _f32(l + c))
            s = s1
        else:  # two_sum_term
            p = _f32(h * xj)
            pe = _f32(h * xj - p)
            s1 = _f32(s + p)
            bb = _f32(s1 - s)
            err = _f32(_f32(s - _f32(s1 - bb)) + _f32(p - bb))
            l = _f32(hl * xj + _f32(l + _f32(err + pe)))
            s = s1
    return s if mode == "fp64" else _f32(s + l)


def _moments(col, val, hi, lo, r0, M, mode):
    rnd = (lambda v: v) if mode == "fp64" else _f32
    mu = np.zeros((M, r0.shape[1]))
    x0 = r0.copy()
    x1 = rnd(0.5 * _row_sums(col, val, hi, lo, x0, mode))
    mu[0] = 0.5 * (x0 * x0).sum(0)
    mu[1] = (x1 * x0).sum(0)
    x, y = x1, x0
    for k in range(2, M // 2 + 1):
        yn = rnd(_row_sums(col, val, hi, lo, x, mode) - y)
        mu[2 * k - 2] = 2 * ((x * x).sum(0) - mu[0])
        mu[2 * k - 1] = 2 * (yn * x).sum(0) - mu[1]
        y, x = x, yn
    return mu


def test_compensated_row_sums_reduce_the_fp32_moment_error():
    h = L.graphene_flake(3000, onsite_modifiers=[L.anderson_disorder(1.0, 3)]).hamiltonian.astype(np.float64)
    n = h.shape[0]
    a, b = 9.5, 0.0
    h2 = ((2.0 / a) * (h - b * sp.identity(n))).tocsr()
    col, val = _ell(h2)
    hi = _f32(val)
    lo = _f32(val - hi)
    rng = np.random.default_rng(7)
    r0 = np.where(rng.integers(0, 2, (n, 2)) == 0, -1.0, 1.0)
    M = 1026
    ref = _moments(col, val, hi, lo, r0, M, "fp64")
    scale = np.abs(ref).max()
    err = {mode: float(np.abs(_moments(col, val, hi, lo, r0, M, mode) - ref).max() / scale)
           for mode in ("fma", "fma_compensated", "two_sum")}
    print(err)
    assert err["fma_compensated"] < err["fma"] / 4
    assert err["two_sum"] < err["fma"] / 4
    assert err["fma_compensated"] < 3 * err["two_sum"]
