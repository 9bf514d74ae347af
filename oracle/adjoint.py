"""Adjoint of the diagonal KPM moments -- NumPy restatement (test infrastructure).

TEST INFRASTRUCTURE ONLY: it checks the GPU adjoint (pybinding_gb300's
kpm_adjoint_diag). Only tests/ import it. pybinding itself has no gradients;
this follows the forward algorithm of the diagonal moments
(cppcore/include/kpm/calc_moments.hpp:35-58 driver, collectors.cpp:6-36
collector, Starter.hpp:55-118 for r1) and differentiates it by hand.

Forward (S = 2 (H - b) / a, the stored optimized matrix; one starter r):
    v0 = r,  v1 = S v0 / 2,  v_k = S v_{k-1} - v_{k-2}        k = 2 .. N   (N = M / 2)
    mu_1 = <v1|v0>,  mu_{2k} = 2 <v_k|v_k> - mu_0,  mu_{2k+1} = 2 <v_{k+1}|v_k> - mu_1
Loss L = sum_n w_n mean_r mu_n(r). With alpha_k = 2 w_{2k} / R (k = 1 .. N-1),
beta_k = 2 w_{2k-1} / R (k = 2 .. N), c1 = (w_1 - sum_{k=2..N} w_{2k-1}) / R, the
adjoint vectors lam_k = dL/dv_k follow the same three-term recursion backwards:
    lam_N = beta_N v_{N-1}
    lam_k = S lam_{k+1} - lam_{k+2} + 2 alpha_k v_k + beta_k v_{k-1} + beta_{k+1} v_{k+1}
and the gradient with respect to the stored entries of S is
    dL/dS = sum_{k=1..N-1} lam_{k+1} v_k^T + (lam_1 / 2 + c1 v0 / 2) v0^T
restricted to the sparsity pattern; dL/dH = (2 / a) dL/dS (a, b frozen).
Forward vectors are recomputed per segment from checkpoints (v_c, v_{c+1})
every `checkpoint` steps, as the GPU does.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def forward_moments(S, r0, M):
    """Averaged diagonal moments (mu_0 unhalved here) of starters r0 (R, n): (M,)."""
    S = sp.csr_matrix(S)
    R = r0.shape[0]
    N = M // 2
    mu = np.zeros(M)
    for r in r0:
        v_prev, v = r, 0.5 * (S @ r)
        m = np.zeros(M)
        m[0] = r @ r
        m[1] = v @ r
        for k in range(1, N):
            v_next = S @ v - v_prev
            m[2 * k] = 2 * (v @ v) - m[0]
            m[2 * k + 1] = 2 * (v_next @ v) - m[1]
            v_prev, v = v, v_next
        mu += m
    return mu / R


def adjoint(S, r0, M, w, checkpoint=0):
    """dL/dS on the pattern of S (CSR, same indices) for L = sum_n w_n mean_r mu_n(r)."""
    S = sp.csr_matrix(S)
    S.sort_indices()
    n = S.shape[0]
    R = r0.shape[0]
    N = M // 2
    w = np.asarray(w, np.float64)
    alpha = np.zeros(N + 2)
    beta = np.zeros(N + 2)
    for k in range(1, N):
        alpha[k] = 2 * w[2 * k] / R
    for k in range(2, N + 1):
        beta[k] = 2 * w[2 * k - 1] / R
    c1 = (w[1] - sum(w[2 * k - 1] for k in range(2, N + 1))) / R
    s = checkpoint if checkpoint > 0 else max(1, int(np.ceil(np.sqrt(N))))
    rows = np.repeat(np.arange(n), np.diff(S.indptr))
    cols = S.indices
    grad = np.zeros(S.nnz)
    for r in r0:
        # forward with checkpoints (v_c, v_{c+1}) at c = 0, s, 2s, ...
        ck = {}
        v_prev, v = r.copy(), 0.5 * (S @ r)
        for k in range(0, N):
            if k % s == 0:
                ck[k] = (v_prev.copy(), v.copy())
            if k + 1 < N:
                v_prev, v = v, S @ v - v_prev
        lam1 = None  # lam_{k+1}
        lam2 = np.zeros(n)  # lam_{k+2}
        starts = sorted([c for c in ck if c + 1 <= N - 1], reverse=True)
        for c in starts:
            kmax = min(c + s, N - 1)
            seg = {c: ck[c][0], c + 1: ck[c][1]}
            for k in range(c + 1, kmax + 1):
                seg[k + 1] = S @ seg[k] - seg[k - 1]
            if lam1 is None:  # lam_N
                lam1 = beta[N] * seg[N - 1]
            for k in range(kmax, c, -1):
                grad += lam1[rows] * seg[k][cols]  # lam_{k+1} v_k^T
                src = 2 * alpha[k] * seg[k] + beta[k] * seg[k - 1] + beta[k + 1] * seg[k + 1]
                lam_k = S @ lam1 - lam2 + src
                lam2, lam1 = lam1, lam_k
        if lam1 is None:  # N == 1: no steps
            lam1 = np.zeros(n)
        u = 0.5 * lam1 + 0.5 * c1 * r
        grad += u[rows] * r[cols]
    return sp.csr_matrix((grad, S.indices.copy(), S.indptr.copy()), shape=S.shape)


def dense_gradient(H, a, b, w):
    """Exact-trace gradient dL/dH for L = sum_n w_n tr(T_n(H~)) / n_sites, H~ = (H - b) / a (dense eigh)."""
    Hd = np.asarray(H.todense() if sp.issparse(H) else H, np.float64)
    n = Hd.shape[0]
    lam, Q = np.linalg.eigh((Hd - b * np.eye(n)) / a)
    lam = np.clip(lam, -1.0, 1.0)
    # d tr T_n(X) / dX = n U_{n-1}(X);  U_{n-1}(x) by its recurrence
    d = np.zeros(n)
    u_prev, u = np.zeros(n), np.ones(n)  # U_{-1}, U_0
    for m in range(1, len(w)):
        d += w[m] * m * u  # u = U_{m-1}
        u_prev, u = u, 2 * lam * u - u_prev
    G = (Q * d) @ Q.T / n
    return G / a
