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

__all__ = ["DiagonalMoments", "ConductivityMoments", "dos", "moments_weights", "kubo_bastin"]


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


class ConductivityMoments:
    """The Kubo-Bastin moments matrix of H(values) for fixed starters, differentiable in ``values``.

    The forward algorithm is ``Core::conductivity``'s (``cppcore/src/kpm/Core.cpp:119-145``):
    mu[m, n] = mean_r <T_m(H~) V_l r, V_r T_n(H~) r>, row and column 0 halved, with the velocity
    operators V = H o (x_i - x_j) of the ``left`` and ``right`` coordinates (``kpm/Moments.cpp:132-155``)
    -- so ``values`` enter through the recursion and through both velocity operators. The
    backward pass is the engine's adjoint of both Chebyshev chains (``kpm_adjoint_conductivity``),
    FP64 and for real Hamiltonians. The scaling (a, b) comes from a fixed energy range.

    pattern: real square CSR matrix (symmetric pattern); fixes the order of ``values``.
    left, right: site coordinates (float32) of the two directions, e.g. ``system.x``.
    starters: (num_vectors, rows) real array, site order (the reference draws Rademacher vectors).
    """

    def __init__(self, pattern, left, right, num_moments, starters, energy_range):
        h = sp.csr_matrix(pattern)
        if h.shape[0] != h.shape[1]:
            raise ValueError("the pattern must be square")
        if np.iscomplexobj(h.data):
            raise ValueError("conductivity gradients need a real Hamiltonian")
        h = h.copy()
        h.sort_indices()
        if energy_range is None or energy_range[0] >= energy_range[1]:
            raise ValueError("a fixed energy_range (min < max) is required: the scaling is not differentiated")
        self.indptr = h.indptr.astype(np.int32)
        self.indices = h.indices.astype(np.int32)
        self.rows = h.shape[0]
        self.num_moments = int(num_moments)
        self.left = np.ascontiguousarray(left, np.float32)
        self.right = np.ascontiguousarray(right, np.float32)
        st = np.atleast_2d(np.asarray(starters, np.float64))
        if st.shape[1] != self.rows:
            raise ValueError("starters must have shape (num_vectors, %d)" % self.rows)
        self.starters = np.ascontiguousarray(st)
        self._cfg = dict(energy_range=tuple(float(x) for x in energy_range), precision="fp64")
        self._engine = None

    @property
    def nnz(self):
        return int(self.indptr[-1])

    def _engine_for(self, values):
        v = np.ascontiguousarray(np.asarray(values, dtype=np.float64))
        if v.shape != (self.nnz,):
            raise ValueError("values must have shape (%d,)" % self.nnz)
        h = sp.csr_matrix((v, self.indices, self.indptr), shape=(self.rows, self.rows))
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

    @property
    def energy_bounds(self):
        """The engine's (min, max) energies (the configured range, as the reference stores it)."""
        if self._engine is None:
            self._engine_for(np.ones(self.nnz))
        return self._engine.energy_bounds(0)[:2]

    def moments(self, values):
        """Forward only (NumPy): mu (M, M), undamped."""
        mu, _, _ = self._engine_for(values).adjoint_conductivity(self.left, self.right, self.num_moments,
                                                                 self.starters)
        return mu

    def gradient(self, values, dl_dmu):
        """Backward only (NumPy): (dL/dvalues per stored entry, dL/d onsite per site) for
        L = sum(dl_dmu * mu)."""
        _, gv, go = self._engine_for(values).adjoint_conductivity(self.left, self.right, self.num_moments,
                                                                  self.starters, np.asarray(dl_dmu, np.float64))
        return gv, go

    def __call__(self, values):
        return _conductivity_fn().apply(values, self)


_CFN = None


def _conductivity_fn():
    global _CFN
    if _CFN is None:
        torch = _torch()

        class ConductivityFn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, values, op):
                ctx.op = op
                ctx.save_for_backward(values)
                return torch.from_numpy(op.moments(values.detach().cpu().numpy())).to(values.device)

            @staticmethod
            def backward(ctx, grad_mu):
                (values,) = ctx.saved_tensors
                gv, _ = ctx.op.gradient(values.detach().cpu().numpy(), grad_mu.detach().cpu().numpy())
                return torch.from_numpy(gv).to(device=values.device, dtype=values.dtype), None

        _CFN = ConductivityFn
    return _CFN


# Boltzmann constant in eV/K, in the reference's float (numeric/constant.hpp)
_KB = float(np.float32(8.6173303e-5))


def kubo_bastin(mu, chemical_potential, scaling, energy_bounds, kernel, temperature=0.0, num_points=1000):
    """Differentiable Kubo-Bastin conductivity (real part) from an UNDAMPED moments matrix
    (torch (M, M) -> (len(chemical_potential),)): the matrix damping g_m g_n (``Kernel.hpp:48-56``)
    and ``reconstruct<KuboBastin>`` (``cppcore/include/kpm/reconstruct.hpp:90-143``) in FP64, as the
    engine's ``calc_conductivity`` computes them: energy samples linspace(min, max, num_points)
    scaled by (a, b), trapezoid weights, Fermi-Dirac occupation (the step function, 1/2 on the
    edge, at T = 0), prefix 4 / a^2. For real moments the real part is
    sigma = sum_mn mu_mn g_m g_n sum_p w_p f(E_p) (T_m(E_p) Re A_n(E_p) + T_n(E_p) Re A_m(E_p))
    / (1 - E_p^2)^2 with A_n(E) = (E - i n sqrt(1 - E^2)) e^{i n acos E}."""
    torch = _torch()
    a, b = scaling
    M = mu.shape[0]
    g = torch.from_numpy(np.asarray(kernel.damping_coefficients(M), np.float64)).to(mu.device)
    mud = mu * g[:, None] * g[None, :]
    emin, emax = energy_bounds
    samples = (emin + (emax - emin) * np.arange(num_points) / (num_points - 1) - b) / a
    samples[-1] = (emax - b) / a
    th = np.arccos(samples)
    sq = np.sqrt(1.0 - samples ** 2)
    n = np.arange(M)
    T = np.cos(np.outer(th, n))
    reA = samples[:, None] * np.cos(np.outer(th, n)) + n[None, :] * sq[:, None] * np.sin(np.outer(th, n))
    k = 1.0 / ((1.0 - samples ** 2) ** 2)
    coeff = (samples.max() - samples.min()) / (2 * num_points)
    w = np.full(num_points, 2.0)
    w[0] = w[-1] = 1.0
    chem = (np.atleast_1d(np.asarray(chemical_potential, np.float64)) - b) / a
    if temperature == 0:
        f = np.where(samples[None, :] < chem[:, None], 1.0, np.where(samples[None, :] > chem[:, None], 0.0, 0.5))
    else:
        f = 1.0 / (1.0 + np.exp((samples[None, :] - chem[:, None]) * (a / (_KB * temperature))))
    omega = (4.0 / (a * a)) * coeff * f * (w * k)[None, :]  # (chem, samples)
    Tt = torch.from_numpy(T).to(mu.device)
    At = torch.from_numpy(reA).to(mu.device)
    s = ((Tt @ mud) * At).sum(1) + ((At @ mud) * Tt).sum(1)  # (samples,)
    return torch.from_numpy(omega).to(mu.device) @ s

