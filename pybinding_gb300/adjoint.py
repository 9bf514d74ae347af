"""Reverse-mode gradients of KPM moments through the GB300 engine (torch.autograd).

pybinding computes no gradients; this module adds them for the diagonal path
(DOS-type moments, ``cpb::kpm`` ``calc_dos``/``moments`` forward algorithm,
``cppcore/include/kpm/calc_moments.hpp:35-58``). The moments

    mu_n = mean_r <r| T_n((H - b) / a) |r>

of a fixed sparsity pattern are a differentiable function of the stored entries
of H; the backward pass is the engine's adjoint Chebyshev recursion
(``kpm_adjoint_diag``) with checkpointed forward vectors. The scaling (a, b) comes
from a fixed energy range and is not differentiated. Real Hamiltonians only.

Example: gradient of a DOS misfit with respect to onsite energies and hoppings
(values of H built from parameters with torch operations)::

    op = DiagonalMoments(pattern, num_moments=1024, starters=r, energy_range=(-9, 9))
    mu = op(values)                      # values: torch tensor, CSR order of `pattern`
    rho = dos(mu, energy, op.scaling, jackson_kernel())
    loss = ((rho - target) ** 2).sum()
    loss.backward()                      # values.grad: dL/dH per stored entry
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

from . import _binding

__all__ = ["DiagonalMoments", "dos", "moments_weights"]


def _torch():
    import torch
    return torch


class DiagonalMoments:
    """Averaged diagonal moments of H(values) for fixed starters, differentiable in ``values``.

    pattern: real square CSR matrix; its (sorted) index structure fixes the order of
        ``values`` (the pattern must be symmetric, as every Hamiltonian's is).
    num_moments: rounded up as the reference does (``round_num_moments``).
    starters: (num_vectors, rows) real array, site order.
    energy_range: (min, max) that fixes the scaling a, b (``Bounds.hpp:11-24``).
    precision: "fp64" (FP64 recursion) or "fp32" (FP32 vectors, FP64 moment sums).
    checkpoint: forward vectors kept every ``checkpoint`` steps and recomputed per segment;
        0 = all of them when they fit in half the free device memory, else sqrt(M/2).
    """

    def __init__(self, pattern, num_moments, starters, energy_range, precision="fp64", checkpoint=0):
        h = sp.csr_matrix(pattern)
        if h.shape[0] != h.shape[1]:
            raise ValueError("the pattern must be square")
        if np.iscomplexobj(h.data):
            raise ValueError("adjoint gradients need a real Hamiltonian")
        h = h.copy()
        h.sort_indices()
        if energy_range is None or energy_range[0] >= energy_range[1]:
            raise ValueError("a fixed energy_range (min < max) is required: the scaling is not differentiated")
        self.indptr = h.indptr.astype(np.int32)
        self.indices = h.indices.astype(np.int32)
        self.rows = h.shape[0]
        self.num_moments = _binding.round_num_moments(int(num_moments))
        self.dtype = np.dtype(np.float64 if precision == "fp64" else np.float32)
        st = np.atleast_2d(np.asarray(starters))
        if st.shape[1] != self.rows:
            raise ValueError("starters must have shape (num_vectors, %d)" % self.rows)
        self.starters = np.ascontiguousarray(st, self.dtype)
        self.checkpoint = int(checkpoint)
        self._cfg = dict(energy_range=tuple(float(x) for x in energy_range), precision=precision)
        self._engine = None

    @property
    def nnz(self):
        return int(self.indptr[-1])

    def matrix(self, values):
        v = np.ascontiguousarray(np.asarray(values, dtype=self.dtype))
        if v.shape != (self.nnz,):
            raise ValueError("values must have shape (%d,)" % self.nnz)
        return sp.csr_matrix((v, self.indices, self.indptr), shape=(self.rows, self.rows))

    def _engine_for(self, values):
        h = self.matrix(values)
        if self._engine is None:
            self._engine = _binding.Engine(h, self._cfg)
        else:
            self._engine.set_hamiltonian(h)
        return self._engine

    @property
    def scaling(self):
        """(a, b) of the fixed energy range."""
        if self._engine is None:
            self._engine_for(np.ones(self.nnz))
        return self._engine.scaling_factors(0)

    def moments(self, values):
        """Forward only (NumPy): averaged moments, float64 (M,)."""
        eng = self._engine_for(values)
        return eng.moments_diag(self.num_moments, self.starters[None], average=True)[0].real.copy()

    def gradient(self, values, dl_dmu):
        """Backward only (NumPy): (dL/dvalues per stored entry, dL/d onsite per site)."""
        eng = self._engine_for(values)
        return eng.adjoint_diag(self.num_moments, self.starters, np.asarray(dl_dmu, np.float64), self.checkpoint)

    def __call__(self, values):
        return _moments_fn().apply(values, self)


_FN = None


def _moments_fn():
    global _FN
    if _FN is None:
        torch = _torch()

        class MomentsFn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, values, op):
                ctx.op = op
                ctx.save_for_backward(values)
                mu = op.moments(values.detach().cpu().numpy())
                return torch.from_numpy(mu).to(values.device)

            @staticmethod
            def backward(ctx, grad_mu):
                (values,) = ctx.saved_tensors
                gv, _ = ctx.op.gradient(values.detach().cpu().numpy(), grad_mu.detach().cpu().numpy())
                return torch.from_numpy(gv).to(device=values.device, dtype=values.dtype), None

        _FN = MomentsFn
    return _FN


def moments_weights(energy, scaling, kernel, num_moments):
    """The linear map moments -> DOS of the engine's ``calc_dos`` (``reconstruct.hpp:16-40``
    with kernel damping, ``Kernel.hpp:21-56``): rho(E) = sum_n W[E, n] mu_n, (len(energy), M)."""
    a, b = scaling
    e = (np.asarray(energy, np.float64) - b) / a
    g = np.asarray(kernel.damping_coefficients(num_moments), np.float64)
    n = np.arange(num_moments)
    t = np.arccos(e)
    return (2.0 / math.pi / a) / np.sqrt(1.0 - e * e)[:, None] * np.cos(n[None, :] * t[:, None]) * g[None, :]


def dos(mu, energy, scaling, kernel):
    """Differentiable DOS from averaged moments (torch tensor (M,) -> (len(energy),))."""
    torch = _torch()
    w = torch.from_numpy(moments_weights(energy, scaling, kernel, mu.shape[0])).to(device=mu.device, dtype=mu.dtype)
    return w @ mu
