"""Adjoint (reverse-mode) gradients of the diagonal KPM moments.

pybinding has no gradients, so the checks are mathematical: the NumPy
restatement of the adjoint (oracle/adjoint.py) is pinned on the CPU against
central finite differences of the forward moments and against the exact-trace
gradient from a dense eigendecomposition; the GPU adjoint is then checked
against that restatement, against finite differences of the FP64 oracle's
moments, and against the dense gradient on a 2,000-site strained sub-flake
traced with all unit vectors.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import adjoint as OA
from pybinding_gb300 import lattice as L

TOL_FP64 = 1e-9


def _strained_flake(num_sites, amplitude=0.05, period=20.0, onsite=None):
    """t_ij = -2.8 exp(-3.37 (d_ij / a_cc - 1)) under a sinusoidal strain field."""
    mods = [L.strained_hopping(L.sinusoidal_strain(amplitude, period))]
    om = [L.anderson_disorder(onsite, 3)] if onsite else []
    return L.graphene_flake(num_sites, hopping_modifiers=mods, onsite_modifiers=om, is_double=True)


def _scaled(h, a, b):
    """S = 2 (H - b) / a with every diagonal entry stored (explicit zeros included)."""
    h = sp.csr_matrix(h, dtype=np.float64)
    n = h.shape[0]
    coo = h.tocoo()
    rows = np.concatenate([coo.row, np.arange(n)])
    cols = np.concatenate([coo.col, np.arange(n)])
    vals = np.concatenate([coo.data * (2.0 / a), np.full(n, -b * 2.0 / a)])
    s = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()  # duplicates summed, zeros kept
    s.sort_indices()
    return s


def _random_symmetric(n, seed):
    rng = np.random.default_rng(seed)
    d = np.zeros((n, n))
    for i in range(n):
        for j in rng.choice(n, 3, replace=False):
            if i != j:
                d[i, j] = d[j, i] = rng.uniform(-1, 1)
    d += np.diag(rng.uniform(-0.5, 0.5, n))
    return sp.csr_matrix(d)


# ---------------------------------------------------------------- CPU: the derivation
def test_oracle_adjoint_matches_finite_differences_and_dense_gradient():
    h = _random_symmetric(40, 3)
    a, b = 1.3 * np.abs(np.linalg.eigvalsh(h.toarray())).max(), 0.1
    s = _scaled(h, a, b)
    rng = np.random.default_rng(5)
    M = 30
    w = rng.normal(size=M)
    r0 = rng.choice([-1.0, 1.0], size=(3, 40))
    g = OA.adjoint(s, r0, M, w)
    for ck in (1, 2, 4, 100):  # checkpoint intervals change nothing
        np.testing.assert_array_equal(OA.adjoint(s, r0, M, w, checkpoint=ck).data, g.data)
    scale = np.abs(g.data).max()
    for e in rng.choice(s.nnz, 12, replace=False):
        sp_, sm_ = s.copy(), s.copy()
        sp_.data[e] += 1e-6
        sm_.data[e] -= 1e-6
        fd = (w @ OA.forward_moments(sp_, r0, M) - w @ OA.forward_moments(sm_, r0, M)) / 2e-6
        assert abs(fd - g.data[e]) <= 1e-8 * scale
    # exact trace: every unit vector as a starter
    gh = OA.adjoint(s, np.eye(40), M, w).toarray() * (2.0 / a)
    gd = OA.dense_gradient(h, a, b, w)
    mask = s.toarray() != 0
    assert np.abs(gh - gd)[mask].max() <= 1e-12 * np.abs(gd[mask]).max()


def test_diagonal_moments_argument_checks():
    from pybinding_gb300.adjoint import DiagonalMoments
    h = _random_symmetric(20, 1)
    with pytest.raises(ValueError, match="real Hamiltonian"):
        DiagonalMoments(h.astype(np.complex128), 30, np.ones((1, 20)), (-3, 3))
    with pytest.raises(ValueError, match="energy_range"):
        DiagonalMoments(h, 30, np.ones((1, 20)), None)
    with pytest.raises(ValueError, match="starters"):
        DiagonalMoments(h, 30, np.ones((1, 19)), (-3, 3))


# ---------------------------------------------------------------- GPU
def _grad_to_matrix(h, gv):
    return sp.csr_matrix((gv, h.indices, h.indptr), shape=h.shape)


@pytest.mark.gpu
@pytest.mark.parametrize("onsite", [None, 0.5])
def test_gpu_adjoint_matches_oracle_adjoint(onsite):
    """FP64 engine gradient per stored entry and per site == the NumPy adjoint on S."""
    from pybinding_gb300 import _native
    m = _strained_flake(3000, onsite=onsite)
    h = sp.csr_matrix(m.hamiltonian, dtype=np.float64)
    h.sort_indices()
    n = h.shape[0]
    rng = np.random.default_rng(7)
    M = 130
    w = rng.normal(size=M)
    r0 = rng.choice([-1.0, 1.0], size=(5, n))
    eng = _native.Engine(h, _native.make_config(energy_range=(-9.5, 9.0), precision="fp64"))
    a, b = eng.scaling_factors()
    gv, go = eng.adjoint_diag(M, r0, w)
    s = _scaled(h, a, b)
    ref = OA.adjoint(s, r0, M, w) * (2.0 / a)
    ref_h = ref.multiply(h != 0).tocsr()  # the entries H stores
    got = _grad_to_matrix(h, gv)
    err = np.abs((got - ref_h).toarray()).max() / np.abs(ref.data).max()
    err_d = np.abs(go - ref.diagonal()).max() / np.abs(ref.data).max()
    print("n=%d entries %.3e onsite %.3e" % (n, err, err_d))
    assert err < TOL_FP64 and err_d < TOL_FP64
    # checkpoint intervals recompute the same vectors: identical gradients
    for ck in (2, 5, M):
        gv2, go2 = eng.adjoint_diag(M, r0, w, checkpoint=ck)
        np.testing.assert_array_equal(gv2, gv)
        np.testing.assert_array_equal(go2, go)


@pytest.mark.gpu
def test_gpu_adjoint_matches_central_differences_of_oracle(oracle):
    """Bond and onsite gradients against central differences of the FP64 oracle's moments."""
    from pybinding_gb300 import _native
    m = _strained_flake(1500, onsite=0.3)
    h = sp.csr_matrix(m.hamiltonian, dtype=np.float64)
    h.sort_indices()
    n = h.shape[0]
    rng = np.random.default_rng(3)
    M = 66
    w = rng.normal(size=M)
    r0 = rng.choice([-1.0, 1.0], size=(3, n))
    rng_e = (-9.5, 9.0)
    eng = _native.Engine(h, _native.make_config(energy_range=rng_e, precision="fp64"))
    a, b = eng.scaling_factors()
    gv, go = eng.adjoint_diag(M, r0, w)

    def loss(hh):
        s = _scaled(hh, a, b)
        mu = oracle.moments_diag(s, r0, M, ell=False, interleaved=False).real.mean(axis=0)
        return float(w @ mu)

    scale = max(np.abs(gv).max(), np.abs(go).max())
    coo = h.tocoo()
    bonds = [k for k in rng.permutation(h.nnz) if coo.row[k] < coo.col[k]][:6]
    eps = 1e-5
    for k in bonds:
        i, j = coo.row[k], coo.col[k]
        dh = sp.csr_matrix(([eps, eps], ([i, j], [j, i])), shape=h.shape)
        fd = (loss(h + dh) - loss(h - dh)) / (2 * eps)
        kt = h.indptr[j] + np.searchsorted(h.indices[h.indptr[j]:h.indptr[j + 1]], i)
        an = gv[k] + gv[kt]
        print("bond (%d,%d): fd %.9e adjoint %.9e" % (i, j, fd, an))
        assert abs(fd - an) <= 1e-6 * scale
    for i in rng.choice(n, 4, replace=False):
        dh = sp.csr_matrix(([eps], ([i], [i])), shape=h.shape)
        fd = (loss(h + dh) - loss(h - dh)) / (2 * eps)
        print("onsite %d: fd %.9e adjoint %.9e" % (i, fd, go[i]))
        assert abs(fd - go[i]) <= 1e-6 * scale


@pytest.mark.gpu
def test_gpu_adjoint_matches_dense_eigh_gradient():
    """Exact trace (all 2,000 unit vectors as starters) on a strained 2k-site sub-flake vs
    the gradient from a dense FP64 eigendecomposition."""
    from pybinding_gb300 import _native
    m = _strained_flake(2000, onsite=0.2)
    h = sp.csr_matrix(m.hamiltonian, dtype=np.float64)
    h.sort_indices()
    n = h.shape[0]
    rng = np.random.default_rng(11)
    M = 66
    w = rng.normal(size=M) / np.arange(1, M + 1)
    eng = _native.Engine(h, _native.make_config(energy_range=(-9.5, 9.0), precision="fp64"))
    a, b = eng.scaling_factors()
    gv, go = eng.adjoint_diag(M, np.eye(n), w)
    gd = OA.dense_gradient(h, a, b, w)
    coo = h.tocoo()
    ref_v = gd[coo.row, coo.col]
    scale = np.abs(gd).max()
    err_v = np.abs(gv - ref_v).max() / scale
    err_d = np.abs(go - np.diag(gd)).max() / scale
    print("n=%d dense eigh: entries %.3e onsite %.3e" % (n, err_v, err_d))
    assert err_v < TOL_FP64 and err_d < TOL_FP64


@pytest.mark.gpu
def test_gpu_adjoint_fp32_close_to_fp64():
    """FP32 recursion (FP32 vectors, FP64 gradient sums over the steps) against the FP64 one on a
    64k-site strained flake (spectrum +-9.11 eV inside the range +-9.5 eV), 1026 moments, 32
    Rademacher vectors: within 1e-5 of the largest entry."""
    from pybinding_gb300 import _native
    m = _strained_flake(64000)
    h = sp.csr_matrix(m.hamiltonian, dtype=np.float64)
    h.sort_indices()
    n = h.shape[0]
    rng = np.random.default_rng(2)
    M = 1024
    Mr = _native.round_num_moments(M)
    w = rng.normal(size=Mr) / np.sqrt(np.arange(1, Mr + 1))
    r0 = rng.choice([-1.0, 1.0], size=(32, n))
    out = {}
    for prec in ("fp64", "fp32"):
        hh = h.astype(np.float64 if prec == "fp64" else np.float32)
        eng = _native.Engine(hh, _native.make_config(energy_range=(-9.5, 9.5), precision=prec))
        out[prec] = eng.adjoint_diag(M, r0, w)
    scale = np.abs(out["fp64"][0]).max()
    err = np.abs(out["fp32"][0] - out["fp64"][0]).max() / scale
    err_d = np.abs(out["fp32"][1] - out["fp64"][1]).max() / scale
    print("fp32 vs fp64 gradient: entries %.3e onsite %.3e" % (err, err_d))
    assert err < 1e-5 and err_d < 1e-5


@pytest.mark.gpu
def test_gpu_adjoint_fp32_at_the_strained_flake_configuration_matches_finite_differences():
    """The adjoint configuration as configured: 256k-site strained graphene (5 % sinusoidal
    strain, period 20 nm, t_ij = -2.8 exp(-3.37 (d/a_cc - 1))), 1024 moments (1026), 32
    Rademacher vectors, FP32 recursion. Gradients of L = sum_n w_n mu_n on sampled bonds and
    sites against central differences of the FP64 recursion's L: within 1e-5 of the largest
    gradient entry."""
    from pybinding_gb300 import _native
    m = _strained_flake(256_000)
    h = sp.csr_matrix(m.hamiltonian, dtype=np.float64)
    h.sort_indices()
    n = h.shape[0]
    rng = np.random.default_rng(6)
    M = 1024
    Mr = _native.round_num_moments(M)
    w = rng.normal(size=Mr) / np.sqrt(np.arange(1, Mr + 1))
    r0 = rng.choice([-1.0, 1.0], size=(32, n))
    rng_e = (-9.5, 9.5)  # the strained flake's spectrum is +-9.11 eV
    e32 = _native.Engine(h.astype(np.float32), _native.make_config(energy_range=rng_e, precision="fp32"))
    gv, go = e32.adjoint_diag(M, r0, w)
    e32.close()
    e64 = _native.Engine(h, _native.make_config(energy_range=rng_e, precision="fp64"))
    gv64, go64 = e64.adjoint_diag(M, r0, w)
    scale = max(np.abs(gv64).max(), np.abs(go64).max())
    full = max(np.abs(gv - gv64).max(), np.abs(go - go64).max()) / scale
    print("256k fp32 adjoint vs fp64 adjoint, all entries: %.3e" % full)

    def loss(values):
        e64.set_hamiltonian(sp.csr_matrix((values, h.indices, h.indptr), shape=h.shape))
        return float(w @ e64.moments_diag(M, r0[None], average=True)[0].real)

    def onsite_loss(i, d):
        hh = (h + sp.csr_matrix(([d], ([i], [i])), shape=h.shape)).tocsr()
        hh.sort_indices()
        e64.set_hamiltonian(hh)
        return float(w @ e64.moments_diag(M, r0[None], average=True)[0].real)

    # central differences with one Richardson step (error O(eps^4): with 1026 moments the
    # eps^2 term of a plain central difference is ~(M eps 2/a)^2 of the derivative)
    def richardson(f, eps):
        d1 = (f(eps) - f(-eps)) / (2 * eps)
        d2 = (f(eps / 2) - f(-eps / 2)) / eps
        return (4 * d2 - d1) / 3

    coo = h.tocoo()
    eps = 4e-5
    worst = 0.0
    for k in [k for k in rng.permutation(h.nnz) if coo.row[k] < coo.col[k]][:6]:
        i, j = coo.row[k], coo.col[k]
        kt = h.indptr[j] + np.searchsorted(h.indices[h.indptr[j]:h.indptr[j + 1]], i)

        def f(d, k=k, kt=kt):
            v = h.data.copy()
            v[k] += d
            v[kt] += d
            return loss(v)
        fd = richardson(f, eps)
        an = gv[k] + gv[kt]
        worst = max(worst, abs(fd - an) / scale)
        print("bond (%d,%d): fd %.9e fp32 adjoint %.9e" % (i, j, fd, an))
    for i in rng.choice(n, 4, replace=False):
        fd = richardson(lambda d, i=i: onsite_loss(i, d), eps)
        worst = max(worst, abs(fd - go[i]) / scale)
        print("onsite %d: fd %.9e fp32 adjoint %.9e" % (i, fd, go[i]))
    e64.close()
    print("largest |fd - adjoint| / max |grad|: %.3e" % worst)
    assert worst <= 1e-5 and full <= 1e-5


@pytest.mark.gpu
def test_torch_autograd_dos_loss():
    """loss(DOS(mu(values))).backward() through torch equals the chain rule done by hand
    with the engine's gradient, and moves the loss as a directional derivative predicts."""
    torch = pytest.importorskip("torch")
    from pybinding_gb300 import jackson_kernel
    from pybinding_gb300.adjoint import DiagonalMoments, dos, moments_weights
    m = _strained_flake(4000, onsite=0.1)
    h = sp.csr_matrix(m.hamiltonian, dtype=np.float64)
    h.sort_indices()
    n = h.shape[0]
    r0 = np.random.default_rng(1).choice([-1.0, 1.0], size=(8, n))
    op = DiagonalMoments(h, 258, r0, (-9.5, 9.0), precision="fp64")
    energy = np.linspace(-7, 7, 41)
    kern = jackson_kernel()
    target = torch.from_numpy(np.exp(-energy ** 2 / 8) * 0.05)
    values = torch.tensor(h.data, dtype=torch.float64, requires_grad=True)
    mu = op(values)
    rho = dos(mu, energy, op.scaling, kern)
    loss = ((rho - target) ** 2).sum()
    loss.backward()
    wmat = moments_weights(energy, op.scaling, kern, op.num_moments)
    dl_drho = 2 * (rho.detach().numpy() - target.numpy())
    gv, _ = op.gradient(h.data, wmat.T @ dl_drho)
    np.testing.assert_allclose(values.grad.numpy(), gv, rtol=0, atol=1e-12 * np.abs(gv).max())
    # directional derivative along a random symmetric perturbation of the values
    rng = np.random.default_rng(4)
    d = sp.csr_matrix((rng.normal(size=h.nnz), h.indices, h.indptr), shape=h.shape)
    d = sp.csr_matrix(d + d.T)
    d.sort_indices()
    assert np.array_equal(d.indices, h.indices)
    eps = 1e-6
    with torch.no_grad():
        lp = ((dos(op(torch.from_numpy(h.data + eps * d.data)), energy, op.scaling, kern) - target) ** 2).sum()
        lm = ((dos(op(torch.from_numpy(h.data - eps * d.data)), energy, op.scaling, kern) - target) ** 2).sum()
    fd = float(lp - lm) / (2 * eps)
    an = float(values.grad.numpy() @ d.data)
    print("directional derivative: fd %.9e adjoint %.9e" % (fd, an))
    assert abs(fd - an) <= 1e-6 * abs(an)


# ---------------------------------------------------------------- conductivity
def _numpy_conductivity_moments(h, left, right, a, b, r0, M):
    """mu[m, n] = mean_r h_m h_n <T_m(H~) V_l r, V_r T_n(H~) r> in NumPy FP64 (Core.cpp:119-145,
    collectors.cpp:82-107; V = H o (x_i - x_j) with float32 coordinate differences)."""
    s = _scaled(h, a, b)
    coo = sp.csr_matrix(h, dtype=np.float64).tocoo()
    dl = (left[coo.row] - left[coo.col]).astype(np.float64)
    dr = (right[coo.row] - right[coo.col]).astype(np.float64)
    vl = sp.csr_matrix((coo.data * dl, (coo.row, coo.col)), shape=h.shape)
    vr = sp.csr_matrix((coo.data * dr, (coo.row, coo.col)), shape=h.shape)

    def chain(start):
        t = [start, 0.5 * (s @ start)]
        for _ in range(2, M):
            t.append(s @ t[-1] - t[-2])
        return np.array(t)

    mu = np.zeros((M, M))
    for r in r0:
        tl = chain(vl @ r)
        u = np.array([vr @ x for x in chain(r)])
        mu += tl @ u.T
    hm = np.ones(M)
    hm[0] = 0.5
    return mu * np.outer(hm, hm) / r0.shape[0]


@pytest.mark.gpu
def test_gpu_conductivity_moments_and_kubo_bastin_match_numpy_and_engine():
    """The conductivity moments matrix of explicit starters (the forward pass of the conductivity
    gradient) equals a NumPy FP64 evaluation of Core::conductivity's moments, and the
    differentiable torch Kubo-Bastin equals the engine's reconstruction of the same moments."""
    torch = pytest.importorskip("torch")
    from pybinding_gb300 import _native, jackson_kernel
    from pybinding_gb300.adjoint import ConductivityMoments, kubo_bastin
    m = _strained_flake(1200, onsite=0.3)
    h = sp.csr_matrix(m.hamiltonian, dtype=np.float64)
    h.sort_indices()
    x = m.system.x
    y = m.system.y
    rng = np.random.default_rng(8)
    r0 = rng.choice([-1.0, 1.0], size=(3, h.shape[0]))
    M = 40
    op = ConductivityMoments(h, x, y, M, r0, (-9.5, 9.0))
    mu = op.moments(h.data)
    a, b = op.scaling
    ref = _numpy_conductivity_moments(h, x, y, a, b, r0, M)
    err = np.abs(mu - ref).max() / np.abs(ref).max()
    print("conductivity moments vs NumPy: %.3e" % err)
    assert err < TOL_FP64
    chem = np.linspace(-1.0, 1.0, 7)
    kern = jackson_kernel()
    sig = kubo_bastin(torch.from_numpy(mu), chem, op.scaling, op.energy_bounds, kern, 0.0, 300).numpy()
    g = kern.damping_coefficients(M)
    eng = _native.Engine(h, _native.make_config(energy_range=(-9.5, 9.0), precision="fp64"))
    ref_sig = eng.kubo_bastin(mu * np.outer(g, g), chem, 0.0, 300).real
    eng.close()
    serr = np.abs(sig - ref_sig).max() / np.abs(ref_sig).max()
    print("torch Kubo-Bastin vs the engine's: %.3e" % serr)
    assert serr < 1e-12


@pytest.mark.gpu
def test_gpu_conductivity_gradient_matches_finite_differences():
    """d sigma / d H through the whole conductivity path -- velocity operators, both Chebyshev
    chains, the moments matrix, damping and Kubo-Bastin -- by the engine's adjoint and torch
    autograd, against central differences (one Richardson step) of the forward conductivity on
    sampled bonds and onsite energies of a strained, disordered flake."""
    torch = pytest.importorskip("torch")
    from pybinding_gb300 import jackson_kernel
    from pybinding_gb300.adjoint import ConductivityMoments, kubo_bastin
    m = _strained_flake(1500, onsite=0.3)
    h = sp.csr_matrix(m.hamiltonian, dtype=np.float64)
    h.sort_indices()
    n = h.shape[0]
    rng = np.random.default_rng(9)
    r0 = rng.choice([-1.0, 1.0], size=(2, n))
    M = 50
    chem = np.array([-0.8, -0.2, 0.3, 1.1])
    c = np.array([1.0, -0.5, 2.0, 0.7])
    kern = jackson_kernel()
    op = ConductivityMoments(h, m.system.x, m.system.x, M, r0, (-9.5, 9.0))
    scaling, bounds = op.scaling, op.energy_bounds

    def loss_t(values):
        return (torch.from_numpy(c) * kubo_bastin(op(values), chem, scaling, bounds, kern, 0.0, 400)).sum()

    values = torch.tensor(h.data, dtype=torch.float64, requires_grad=True)
    loss_t(values).backward()
    gv = values.grad.numpy().copy()
    # the onsite disorder stores every diagonal entry: onsite gradients are those entries
    diag_pos = np.array([h.indptr[i] + np.searchsorted(h.indices[h.indptr[i]:h.indptr[i + 1]], i) for i in range(n)])
    assert np.array_equal(h.indices[diag_pos], np.arange(n))
    _, go = op.gradient(h.data, np.zeros((M, M)))
    assert go.shape == (n,) and not np.any(go)

    def loss_np(v, o=op):
        with torch.no_grad():
            return float((torch.from_numpy(c) * kubo_bastin(torch.from_numpy(o.moments(v)), chem, scaling, bounds,
                                                              kern, 0.0, 400)).sum())

    def richardson(f, eps):
        d1 = (f(eps) - f(-eps)) / (2 * eps)
        d2 = (f(eps / 2) - f(-eps / 2)) / eps
        return (4 * d2 - d1) / 3

    scale = np.abs(gv).max()
    coo = h.tocoo()
    eps = 1e-4
    worst = 0.0
    for k in [k for k in rng.permutation(h.nnz) if coo.row[k] < coo.col[k]][:6]:
        i, j = coo.row[k], coo.col[k]
        kt = h.indptr[j] + np.searchsorted(h.indices[h.indptr[j]:h.indptr[j + 1]], i)

        def f(d, k=k, kt=kt):
            v = h.data.copy()
            v[k] += d
            v[kt] += d
            return loss_np(v)
        fd = richardson(f, eps)
        an = gv[k] + gv[kt]
        worst = max(worst, abs(fd - an) / scale)
        print("bond (%d,%d): fd %.9e adjoint %.9e" % (i, j, fd, an))
    for i in rng.choice(n, 4, replace=False):
        def fo(d, i=i):
            v = h.data.copy()
            v[diag_pos[i]] += d
            return loss_np(v)
        fd = richardson(fo, eps)
        worst = max(worst, abs(fd - gv[diag_pos[i]]) / scale)
        print("onsite %d: fd %.9e adjoint %.9e" % (i, fd, gv[diag_pos[i]]))
    print("largest |fd - adjoint| / max |grad|: %.3e" % worst)
    assert worst < 1e-6
