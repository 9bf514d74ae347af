"""GPU parity: the CUDA engine (through the C ABI) against the oracle, the
reference's FP64 NumPy KPM, and the reference's golden arrays.

Error measure for moments: max_n |mu_n - mu_n^ref| / max_n |mu_n^ref|.
Tolerances: FP64 recursion <= 1e-10 (the FP64 accuracy target); FP32 recursion
vectors with FP64 moment sums <= 1e-5 at these sizes (the measured error is
printed); reconstructed functions against the reference goldens at the
reference's own test tolerances.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from pybinding_gb300 import _native, kpm, kpm_batch, lattice as L, lorentz_kernel
from tests import models as TM

pytestmark = pytest.mark.gpu


def rel_err(got, ref):
    return float(np.max(np.abs(np.asarray(got) - np.asarray(ref))) / np.max(np.abs(ref)))


@pytest.mark.parametrize("tag", ["c128", "f64"])
def test_fp64_moments_match_reference_python_impl(python_impl, tag):
    """FP64 recursion == reference _PythonImpl (chebyshev.py:498-520) on identical starters, <= 1e-10."""
    d = python_impl
    n = d[tag + "_indptr"].size - 1
    h = sp.csr_matrix((d[tag + "_data"], d[tag + "_indices"], d[tag + "_indptr"]), shape=(n, n))
    ref = d[tag + "_moments"]
    eng = _native.Engine(h, _native.make_config(energy_range=tuple(d[tag + "_bounds"])))
    assert eng.scaling_factors() == tuple(d[tag + "_ab"])
    got = eng.moments_diag(ref.shape[1], d[tag + "_starters"][None])[0]
    assert got.shape == ref.shape
    err = rel_err(got, ref)
    print("fp64 moment error vs _PythonImpl [%s]: %.3e" % (tag, err))
    assert err <= 1e-10
    # the same vectors one at a time (K = 1 kernel shape) agree too
    one = eng.moments_diag(ref.shape[1], d[tag + "_starters"][1:2][None])[0, 0]
    assert rel_err(one, ref[1]) <= 1e-10


def _disordered_flake(n_sites, seed, dtype=np.float32):
    m = L.graphene_flake(n_sites, onsite_modifiers=[L.anderson_disorder(1.0, seed)])
    return m.hamiltonian.astype(dtype)


@pytest.mark.parametrize("nvec", [64, 13, 3])
def test_fp32_batched_moments_vs_fp64_oracle(oracle, nvec):
    """FP32 vectors + FP64 moment sums against the FP64 oracle on the same H and starters."""
    h = _disordered_flake(6000, 3)
    rng = (-9.0, 9.0)
    M = 514
    a, b = oracle.scale(*rng)
    starters = oracle.random_starters(h.shape[0], nvec, np.float32)
    eng = _native.Engine(h, _native.make_config(energy_range=rng))
    got = eng.moments_diag(M, starters[None])[0]
    r = oracle.optimize(h.astype(np.float64), [0], [0], a, b)
    st = oracle.reorder_vector(starters.astype(np.float64), r["reorder_map"])
    ref = oracle.moments_diag(r["h2"], st, M, slices=r["slices"])
    err = rel_err(got, ref)
    print("fp32-recursion moment error vs fp64 oracle (nvec=%d, M=%d): %.3e" % (nvec, M, err))
    assert err <= 1e-5
    # FP64 mode of the same engine meets the FP64 bar
    eng64 = _native.Engine(h, _native.make_config(energy_range=rng, precision="fp64"))
    got64 = eng64.moments_diag(M, starters[None])[0]
    assert rel_err(got64, ref) <= 1e-10


def test_complex_fp32_moments_vs_fp64_oracle(oracle):
    m = L.graphene_flake(4000, hopping_modifiers=[L.constant_magnetic_field(100)], is_complex=True)
    h = m.hamiltonian
    rng = (-8.7, 8.7)
    a, b = oracle.scale(*rng)
    M = 258
    starters = oracle.random_starters(h.shape[0], 8, np.complex64)
    got = _native.Engine(h, _native.make_config(energy_range=rng)).moments_diag(M, starters[None])[0]
    r = oracle.optimize(h.astype(np.complex128), [0], [0], a, b)
    ref = oracle.moments_diag(r["h2"], oracle.reorder_vector(starters.astype(np.complex128), r["reorder_map"]), M,
                              slices=r["slices"])
    err = rel_err(got, ref)
    print("c64-recursion moment error vs c128 oracle: %.3e" % err)
    assert err <= 1e-5


@pytest.mark.parametrize("name", list(TM.DOS_MODELS))
def test_dos_matches_reference_golden(baselines, name):
    """tests/test_kpm.py:146-165 through the pb.kpm-compatible API (rtol 1e-3)."""
    kind, size = TM.DOS_MODELS[name]
    model = TM.graphene(kind, size)
    energy = np.linspace(0, 2, 25)
    for cfg in [dict(optimal_size=False, interleaved=False), dict(optimal_size=True, interleaved=True)]:
        k = kpm(model, kernel=lorentz_kernel(), silent=True, matrix_format="ELL", **cfg)
        dos = k.calc_dos(energy, broadening=0.15)
        np.testing.assert_allclose(dos.data, baselines["dos[%s]" % name], rtol=1e-3, atol=1e-6)


@pytest.mark.parametrize("name", list(TM.LDOS_MODELS))
def test_ldos_matches_reference_golden(baselines, name):
    """tests/test_kpm.py:25-47 (rtol 1e-3, atol 1e-6)"""
    kind, size = TM.LDOS_MODELS[name]
    model = TM.graphene(kind, size)
    energy = np.linspace(0, 2, 25)
    for cfg in [dict(matrix_format="CSR", optimal_size=False, interleaved=False),
                dict(matrix_format="CSR", optimal_size=True, interleaved=False),
                dict(matrix_format="ELL", optimal_size=True, interleaved=True)]:
        k = kpm(model, kernel=lorentz_kernel(), silent=True, **cfg)
        ldos = k.calc_ldos(energy, broadening=0.15, position=[0, 0.07], reduce=False)
        np.testing.assert_allclose(ldos.data, baselines["ldos[%s]" % name], rtol=1e-3, atol=1e-6)


def test_multi_orbital_ldos_matches_reference_golden(baselines):
    """The ldos[mos2] golden of tests/test_kpm.py:22-47: three-band MoS2 (three orbitals per site),
    LDOS of the site nearest (0, 0.07), reduce=False gives one column per orbital and reduce=True
    their sum (KPM.cpp:55-65); Lorentz kernel, rtol 1e-3, atol 1e-6, every configuration."""
    m = L.build_tmd_3band(L.rectangle(6), "MoS2")
    energy = np.linspace(0, 2, 25)
    expected = baselines["ldos[mos2]"]
    for cfg in [dict(matrix_format="CSR", optimal_size=False, interleaved=False),
                dict(matrix_format="CSR", optimal_size=True, interleaved=False),
                dict(matrix_format="CSR", optimal_size=False, interleaved=True),
                dict(matrix_format="ELL", optimal_size=True, interleaved=True)]:
        k = kpm(m, kernel=lorentz_kernel(), silent=True, **cfg)
        ldos = k.calc_ldos(energy, broadening=0.15, position=[0, 0.07], reduce=False)
        assert ldos.data.shape == (25, 3)
        np.testing.assert_allclose(ldos.data, expected, rtol=1e-3, atol=1e-6)
        summed = k.calc_ldos(energy, broadening=0.15, position=[0, 0.07]).data
        np.testing.assert_allclose(summed, ldos.data.sum(axis=1), rtol=1e-12, atol=0)


def test_ldos_equals_oracle_and_multi_index(oracle):
    """Several LDOS columns in one batch; each equals the oracle's Core::ldos."""
    m = TM.graphene("const_potential", 6)
    h = m.hamiltonian.astype(np.float64)
    n = h.shape[0]
    idx = [n // 2, n // 4, n // 2, 7, n - 3]
    energy = np.linspace(-3, 3, 31)
    k = kpm(L.Model(h, m.system), energy_range=(-9, 9), kernel=lorentz_kernel())
    got = k.impl.engine.calc_ldos(idx, energy, 0.2)
    ref = oracle.core_ldos(h, idx, energy, 0.2, energy_range=(-9, 9), kernel="lorentz")
    # the reference's 2/pi prefactor is a float constant (reconstruct.hpp:27); the engine uses exact pi
    assert rel_err(got, ref) < 1e-7
    np.testing.assert_allclose(got[:, 0], got[:, 2], rtol=1e-12)


def test_greens_function(oracle):
    """cppcore/tests/test_kpm.cpp:217-260: LDOS = -Im G_ii / pi; G(i,[j..])[0] = G(j,i) for real H;
    equal to the oracle's Core::greens_vector."""
    m = TM.cpp_fixture_model()
    h = m.hamiltonian.astype(np.float64)
    n = h.shape[0]
    i, j = n // 2, n // 4
    energy = np.linspace(-0.3, 0.3, 10)
    k = kpm(L.Model(h, m.system))
    gs = k.calc_greens(i, [j, j + 1, j + 2], energy, 0.8)
    assert len(gs) == 3
    g = k.calc_greens(j, i, energy, 0.8)
    np.testing.assert_allclose(gs[0], g, rtol=1e-6, atol=1e-9)
    g_ii = k.calc_greens(i, i, energy, 0.8)
    ldos = k.impl.engine.calc_ldos([i], energy, 0.8)[:, 0]
    np.testing.assert_allclose(ldos, -g_ii.imag / np.pi, rtol=1e-9, atol=1e-12)
    emin, emax = k.impl.energy_bounds
    cfg = dict(energy_range=(np.float32(emin), np.float32(emax)))
    eng = _native.Engine(h, _native.make_config(**cfg))
    got = eng.calc_greens(i, [j, j + 1, j + 2], energy, 0.8)
    ref = oracle.core_greens(h, i, [j, j + 1, j + 2], energy, 0.8, **cfg)
    assert rel_err(got, ref) < 1e-9


def test_moments_api(oracle):
    """tests/test_kpm.py:50-84 (moments == manual LDOS) and KPM.cpp:19-53 errors."""
    m = TM.graphene("pristine", 5)
    h = m.hamiltonian.astype(np.float64)
    n = h.shape[0]
    cfg = dict(energy_range=(-9.0, 9.0))
    k = kpm(L.Model(h, m.system), **cfg)
    alpha = np.zeros(n)
    alpha[n // 3] = 1
    mom = k.moments(100, alpha)
    ref = oracle.core_moments(h, 100, alpha, **cfg)
    assert rel_err(mom, ref) < 1e-10
    rng = np.random.default_rng(1)
    beta = rng.standard_normal(n)
    op = sp.random(n, n, density=0.01, random_state=2, format="csr")
    got = k.moments(64, alpha, beta, op)
    ref = oracle.core_moments(h, 64, alpha, beta, op, **cfg)
    assert rel_err(got, ref) < 1e-10
    got = k.moments(64, alpha, None, op)
    ref = oracle.core_moments(h, 64, alpha, None, op, **cfg)
    assert rel_err(got, ref) < 1e-10
    with pytest.raises(RuntimeError, match="Size mismatch"):
        k.moments(10, [1, 2, 3])
    with pytest.raises(RuntimeError, match="Hamiltonian is real, but the given argument 'alpha' is complex"):
        k.moments(10, 1j * alpha)


def test_ragged_batch_equals_single_systems(oracle):
    """A ragged batch of uneven flakes gives each flake's own moments and DOS."""
    hs = [_disordered_flake(n, s, np.float64) for n, s in ((1500, 1), (3700, 2), (800, 3))]
    models = [L.Model(h, None) for h in hs]
    rng = (-9.0, 9.0)
    nvec, M = 8, 130
    starters = [oracle.random_starters(h.shape[0], nvec, np.float64) for h in hs]
    batch = kpm_batch(models, energy_range=rng)
    flat = np.concatenate([s.ravel() for s in starters])
    a, b = oracle.scale(*rng)
    moms = batch.engine.moments_diag(M, flat)
    for s, h in enumerate(hs):
        r = oracle.optimize(h, [0], [0], a, b)
        ref = oracle.moments_diag(r["h2"], oracle.reorder_vector(starters[s], r["reorder_map"]), M,
                                  slices=r["slices"])
        assert rel_err(moms[s], ref) <= 1e-10
    energy = np.linspace(-2, 2, 11)
    dos = batch.calc_dos(energy, 0.2, num_random=2)
    for s, h in enumerate(hs):
        ref, _ = oracle.core_dos(h, energy, 0.2, 2, energy_range=rng)
        np.testing.assert_allclose(dos[s].data, ref, rtol=1e-6, atol=1e-10)


def test_lanczos_bounds_and_multi_system():
    """FP64 GPU Lanczos: extremes within the convergence target, per system of a batch."""
    hs = [_disordered_flake(n, s, np.float64) for n, s in ((300, 4), (700, 5))]
    batch = kpm_batch([L.Model(h, None) for h in hs])
    for s, h in enumerate(hs):
        mn, mx, loops = batch.engine.energy_bounds(s)
        ev = np.linalg.eigvalsh(h.toarray())
        assert mn == pytest.approx(ev[0], rel=2e-3) and mx == pytest.approx(ev[-1], rel=2e-3)
        assert 0 < loops < 1000


def test_minimum_moments_and_single_row():
    h = sp.csr_matrix(np.array([[0.5]]))
    eng = _native.Engine(h, _native.make_config(energy_range=(-1.0, 1.0)))
    mu = eng.moments_diag(2, np.ones((1, 1, 1)))[0, 0]
    assert mu.shape == (2,)
    a, b = eng.scaling_factors()
    assert mu[0] == pytest.approx(0.5) and mu[1].real == pytest.approx((0.5 - b) / a)


def test_report_and_stats():
    m = TM.graphene("const_potential", 8)
    k = kpm(m, kernel=lorentz_kernel())
    k.calc_dos(np.linspace(-1, 1, 5), 0.2, 2)
    s = k.stats
    assert s.num_moments > 0 and s.moments_time > 0 and s.eps > 0
    r = k.report(shortform=True)
    assert "eps" in r and r.count("[") >= 3


@pytest.mark.parametrize("name", list(TM.COND_MODELS))
def test_conductivity_matches_reference_golden(baselines, name):
    """tests/test_kpm.py:176-197 (energy_range [-9, 9], Lorentz, T = 0, 200 points; rtol 1e-2, atol 1e-5)"""
    kind, size = TM.COND_MODELS[name]
    model = TM.graphene(kind, size)
    energy = np.linspace(-2, 2, 25)
    for cfg in [dict(optimal_size=False, interleaved=False), dict(optimal_size=True, interleaved=True)]:
        k = kpm(model, energy_range=[-9, 9], kernel=lorentz_kernel(), silent=True, matrix_format="ELL", **cfg)
        sigma = k.calc_conductivity(energy, broadening=0.5, temperature=0, num_points=200)
        np.testing.assert_allclose(sigma.data, baselines["conductivity[%s]" % name], rtol=1e-2, atol=1e-5)


def test_conductivity_fp64_equals_oracle(oracle):
    """FP64 Kubo-Bastin (dense moments + mu_mn GEMM + reconstruction) against the oracle's Core::conductivity."""
    m = TM.graphene("magnetic_field", 6)
    h = m.hamiltonian.astype(np.complex128)
    x, y = m.system.x, m.system.y
    chem = np.linspace(-1.9, 2.1, 9)
    cfg = dict(energy_range=(-9.0, 9.0), kernel="jackson")
    eng = _native.Engine(h, _native.make_config(**cfg))
    for left, right, nrand in ((x, x, 3), (x, y, 2)):
        got = eng.calc_conductivity(left, right, chem, 0.6, 0.0, nrand, 100)
        ref = oracle.core_conductivity(h, left, right, chem, 0.6, 0.0, nrand, 100, matrix_format="ELL",
                                       optimal_size=False, interleaved=False, **cfg)
        err = rel_err(got, ref)
        print("conductivity fp64 vs oracle: %.3e" % err)
        assert err < 1e-9


@pytest.mark.parametrize("fuse", [1, 2])
@pytest.mark.parametrize("dtype,nvec,tol", [(np.float32, 64, 1e-5), (np.float64, 8, 1e-10),
                                            (np.complex128, 8, 1e-10), (np.complex64, 4, 1e-5)])
def test_one_and_two_steps_per_launch(oracle, fuse, dtype, nvec, tol):
    """Single-step and fused two-step launches both match the FP64 oracle (ragged batch of 2 flakes)."""
    hs = [_disordered_flake(n, s, np.float64) for n, s in ((20000, 8), (9000, 9))]
    if np.iscomplexobj(np.zeros(1, dtype)):
        hs = [(h + 1j * sp.triu(h, 1) * 0.1 - 1j * sp.tril(h, -1) * 0.1).tocsr() for h in hs]
    hs = [h.astype(dtype) for h in hs]
    rng = (-9.5, 9.5)
    M = 258
    a, b = oracle.scale(*rng)
    starters = [oracle.random_starters(h.shape[0], nvec, dtype) for h in hs]
    batch = kpm_batch([L.Model(h, None) for h in hs], energy_range=rng, fuse_steps=fuse)
    moms = batch.engine.moments_diag(M, np.concatenate([st.ravel() for st in starters]))
    assert batch.engine.stats().num_moments == M
    for s, h in enumerate(hs):
        h64 = h.astype(np.complex128 if np.iscomplexobj(h.data) else np.float64)
        r = oracle.optimize(h64, [0], [0], a, b)
        ref = oracle.moments_diag(r["h2"], oracle.reorder_vector(starters[s].astype(h64.dtype), r["reorder_map"]), M,
                                  slices=r["slices"])
        err = rel_err(moms[s], ref)
        print("fuse=%d %s nvec=%d system %d: %.3e" % (fuse, np.dtype(dtype).name, nvec, s, err))
        assert err <= tol


@pytest.mark.parametrize("name", sorted(TM.COND_MODELS))
def test_conductivity_tensor_core_gemm_matches_reference_golden(baselines, name):
    """The tensor-core moments GEMM against the same goldens as the FP64 one (tests/test_kpm.py:176-197)."""
    kind, size = TM.COND_MODELS[name]
    model = TM.graphene(kind, size)
    energy = np.linspace(-2, 2, 25)
    k = kpm(model, energy_range=[-9, 9], kernel=lorentz_kernel(), silent=True, moments_gemm="tensor")
    sigma = k.calc_conductivity(energy, broadening=0.5, temperature=0, num_points=200)
    np.testing.assert_allclose(sigma.data, baselines["conductivity[%s]" % name], rtol=1e-2, atol=1e-5)


@pytest.mark.parametrize("dtype,precision", [(np.complex128, "fp64"), (np.float64, "fp64"),
                                             (np.complex64, "fp32"), (np.float32, "fp32")])
def test_conductivity_tensor_core_gemm_matches_fp64_gemm(oracle, dtype, precision):
    """gemm_mode 1 (tcgen05 TF32 three-product split of FP32 planes) against gemm_mode 0 (FP64
    CUDA cores) on the same engine, and against the FP64 oracle: sigma within 2e-5 of max |sigma|.
    The model is large enough for several 128 x 128 tiles (M = 276 moments) and long slices of
    I = rows x vectors (3 random vectors of ~5,500 sites)."""
    m = TM.graphene("magnetic_field" if np.iscomplexobj(np.zeros(1, dtype)) else "const_potential", 12)
    h = m.hamiltonian.astype(dtype)
    x, y = m.system.x, m.system.y
    chem = np.linspace(-2.5, 2.5, 21)
    cfg = dict(energy_range=(-9.0, 9.0), kernel="jackson", precision=precision)
    eng = _native.Engine(h, _native.make_config(**cfg))
    fp64 = eng.calc_conductivity(x, y, chem, 0.08, 0.0, 3, 200, gemm_mode=0)
    tc = eng.calc_conductivity(x, y, chem, 0.08, 0.0, 3, 200, gemm_mode=1)
    assert eng.stats().num_moments > 256
    err = rel_err(tc, fp64)
    print("%s %s: n=%d M=%d  tensor vs fp64 gemm %.3e" % (np.dtype(dtype).name, precision, h.shape[0],
                                                       eng.stats().num_moments, err))
    assert err < 2e-5
    if precision == "fp64":
        h64 = h.astype(np.complex128 if np.iscomplexobj(h.data) else np.float64)
        ref = oracle.core_conductivity(h64, x, y, chem, 0.08, 0.0, 3, 200, matrix_format="ELL",
                                       optimal_size=True, interleaved=True, energy_range=(-9.0, 9.0),
                                       kernel="jackson")
        err_o = rel_err(tc, ref)
        print("  tensor vs oracle %.3e" % err_o)
        assert err_o < 2e-5


@pytest.mark.parametrize("dtype,nvec", [(np.float64, 8), (np.float32, 64), (np.complex128, 1)])
def test_repeated_calls_replay_the_recursion_graph(dtype, nvec):
    """From the second call on, an engine replays its captured recursion (a CUDA graph). New
    starters, and new values after set_hamiltonian (same sizes, same device buffers), must give
    what a fresh engine gives."""
    h1, h2 = (_disordered_flake(20000, s, np.float64).astype(dtype) for s in (3, 4))
    cfg = dict(energy_range=(-9.5, 9.5))
    rng = np.random.default_rng(0)
    M = 258
    eng = _native.Engine(h1, _native.make_config(**cfg))

    def starters():
        st = np.where(rng.integers(0, 2, (nvec, h1.shape[0])) == 0, -1.0, 1.0)
        return st.astype(dtype)[None]

    def fresh(h, st):
        e = _native.Engine(h, _native.make_config(**cfg))
        out = e.moments_diag(M, st)
        e.close()
        return out

    tol = 1e-12 if np.dtype(dtype) in (np.dtype(np.float64), np.dtype(np.complex128)) else 1e-5
    for _ in range(3):
        st = starters()
        assert rel_err(eng.moments_diag(M, st), fresh(h1, st)) < tol
    eng.set_hamiltonian(h2)
    for _ in range(2):
        st = starters()
        assert rel_err(eng.moments_diag(M, st), fresh(h2, st)) < tol


@pytest.mark.parametrize("dtype,nvec", [(np.float32, 64), (np.float32, 16), (np.float64, 8)])
def test_first_call_gives_the_moments_of_later_calls(dtype, nvec):
    """The first call on a new shape times its launch options on its own first steps, then
    starts the recursion over with the chosen one: its moments equal later calls' up to the
    order of the FP64 atomic adds (FP32 partial sums over other tiles would differ by ~1e-7)."""
    h = _disordered_flake(17011, 9, np.float64).astype(dtype)  # a size no other test uses
    rng = np.random.default_rng(1)
    st = np.where(rng.integers(0, 2, (nvec, h.shape[0])) == 0, -1.0, 1.0).astype(dtype)[None]
    eng = _native.Engine(h, _native.make_config(energy_range=(-9.5, 9.5)))
    first = eng.moments_diag(514, st)
    again = eng.moments_diag(514, st)
    eng.close()
    err = rel_err(first, again)
    print("first vs later call (%s, %d vectors): %.3e" % (np.dtype(dtype).name, nvec, err))
    assert err < 1e-12


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-10), (np.complex64, 1e-5)])
def test_complex_vectors_with_real_valued_hamiltonian(oracle, dtype, tol):
    """A real lattice stored as complex (so that random-phase starters apply, as the 60k-site
    FP64 DOS configuration does): the diagonal step then multiplies by the real values only.
    Moments against the FP64 oracle on the same complex H and starters; a field breaks the
    real-valuedness and takes the complex-value path, checked the same way."""
    for field in (None, 50.0):
        mods = [L.constant_magnetic_field(field)] if field else []
        m = L.graphene_flake(8000, hopping_modifiers=mods, onsite_modifiers=[L.anderson_disorder(0.5, 4)],
                             is_complex=True)
        h = m.hamiltonian.astype(dtype)
        assert (np.abs(h.data.imag).max() == 0) == (field is None)
        rng = (-9.5, 9.5)
        a, b = oracle.scale(*rng)
        M = 258
        starters = oracle.random_starters(h.shape[0], 8, dtype)
        got = _native.Engine(h, _native.make_config(energy_range=rng)).moments_diag(M, starters[None])[0]
        r = oracle.optimize(h.astype(np.complex128), [0], [0], a, b)
        ref = oracle.moments_diag(r["h2"], oracle.reorder_vector(starters.astype(np.complex128), r["reorder_map"]), M,
                                  slices=r["slices"])
        err = rel_err(got, ref)
        print("%s field=%s: %.3e" % (np.dtype(dtype).name, field, err))
        assert err <= tol


def test_disconnected_system(oracle):
    """One system made of two flakes that share no bond plus a site with no entries at all: the
    breadth-first reorder must cover every component (the reference assumes a connected graph).
    Moments against a plain FP64 NumPy recursion on the unreordered matrix; LDOS of a site in the
    second flake equals the LDOS of that flake alone; bit-exact against the oracle's reorder."""
    h1 = _disordered_flake(3000, 1, np.float64)
    h2 = _disordered_flake(2000, 2, np.float64)
    h = sp.block_diag([h1, sp.csr_matrix((1, 1)), h2], format="csr")
    h.sort_indices()
    n = h.shape[0]
    rng = (-9.5, 9.5)
    a, b = oracle.scale(*rng)
    M = 66
    rs = np.random.default_rng(3)
    st = np.where(rs.integers(0, 2, (4, n)) == 0, -1.0, 1.0)
    eng = _native.Engine(h, _native.make_config(energy_range=rng))
    got = eng.moments_diag(M, st[None])[0]
    ht = ((h - b * sp.identity(n)) / a).tocsr()
    ref = np.zeros((4, M))
    for v in range(4):
        r0 = st[v]
        r1 = ht @ r0
        ref[v, 0], ref[v, 1] = r0 @ r0, r1 @ r0
        for k in range(2, M):
            r0, r1 = r1, 2 * (ht @ r1) - r0
            ref[v, k] = r1 @ st[v]
    ref[:, 0] *= 0.5  # the collectors store mu_0 halved
    assert rel_err(got.real, ref) < 1e-12
    energy = np.linspace(-3, 3, 21)
    site = h1.shape[0] + 1 + 100  # in the second flake
    ldos = eng.calc_ldos([site], energy, 0.2)[:, 0]
    alone = _native.Engine(h2, _native.make_config(energy_range=rng)).calc_ldos([100], energy, 0.2)[:, 0]
    np.testing.assert_allclose(ldos, alone, rtol=1e-10, atol=1e-12)
    r = oracle.optimize(h, [site], [site], a, b)
    opt = eng.optimized_hamiltonian([site], [site])
    assert np.array_equal(opt["reorder_map"], r["reorder_map"])


def test_conductivity_zero_temperature_on_a_sample_energy(oracle):
    """At T = 0 a chemical potential that coincides with an energy sample (here mu = -1.0 and
    linspace(-9, 9, 1000) holds -1.0 exactly) makes the reference's Fermi factor 0 * inf = NaN;
    the engine uses the step function with 1/2 on the edge: finite, and equal to the oracle
    everywhere else."""
    m = TM.graphene("magnetic_field", 6)
    h = m.hamiltonian.astype(np.complex128)
    x = m.system.x
    cfg = dict(energy_range=(-9.0, 9.0), kernel="jackson")
    eng = _native.Engine(h, _native.make_config(**cfg))
    chem = np.array([-1.0, -0.987, 0.5])
    got = eng.calc_conductivity(x, x, chem, 0.6, 0.0, 2, 1000)
    assert np.all(np.isfinite(got))
    ref = oracle.core_conductivity(h, x, x, chem, 0.6, 0.0, 2, 1000, matrix_format="ELL", optimal_size=False,
                                   interleaved=False, **cfg)
    assert np.isnan(ref[0])  # the reference's behaviour at this point
    assert rel_err(got[1:], ref[1:]) < 1e-9
    near = eng.calc_conductivity(x, x, np.array([-1.0 - 1e-9, -1.0 + 1e-9]), 0.6, 0.0, 2, 1000)
    assert min(near.real) - 1e-9 * abs(near.real).max() <= got[0].real <= max(near.real) + 1e-9 * abs(near.real).max()


@pytest.mark.parametrize("gemm_mode", [0, 1])
def test_conductivity_in_two_parts(oracle, gemm_mode):
    """kpm_conductivity_moments + damping + kpm_kubo_bastin == kpm_calc_conductivity, and (FP64
    GEMM) equals the oracle's Core::conductivity."""
    m = TM.graphene("magnetic_field", 6)
    h = m.hamiltonian.astype(np.complex128)
    x, y = m.system.x, m.system.y
    cfg = dict(energy_range=(-9.0, 9.0), kernel="jackson")
    eng = _native.Engine(h, _native.make_config(**cfg))
    chem = np.linspace(-1.9, 2.1, 9)
    whole = eng.calc_conductivity(x, y, chem, 0.6, 0.0, 2, 100, gemm_mode=gemm_mode)
    M = eng.stats().num_moments
    mu = eng.conductivity_moments(x, y, M, 2, gemm_mode=gemm_mode)
    g = _native.damping_coefficients("jackson", 4.0, M)
    parts = eng.kubo_bastin(mu * g[:, None] * g[None, :], chem, 0.0, 100)
    assert rel_err(parts, whole) < 1e-12
    if gemm_mode == 0:
        ref = oracle.core_conductivity(h, x, y, chem, 0.6, 0.0, 2, 100, matrix_format="ELL", optimal_size=False,
                                       interleaved=False, **cfg)
        assert rel_err(parts, ref) < 1e-9


def test_engines_on_two_host_threads_agree_with_one_thread():
    """ctypes releases the GIL around engine calls: two engines driven from two host threads at
    once (shared launch caches, process-wide tuning cache) give the moments of one-by-one calls."""
    import threading
    hs = [_disordered_flake(n, 30 + i, np.float64) for i, n in enumerate((7001, 5003))]
    starters = [np.where(np.random.default_rng(i).integers(0, 2, (8, h.shape[0])) == 0, -1.0, 1.0)[None]
                for i, h in enumerate(hs)]
    cfg = dict(energy_range=(-9.5, 9.5))
    ref = [_native.Engine(h, _native.make_config(**cfg)).moments_diag(258, st) for h, st in zip(hs, starters)]
    out = [None, None]
    errors = []

    def run(i):
        try:
            eng = _native.Engine(hs[i], _native.make_config(**cfg))
            for _ in range(3):
                out[i] = eng.moments_diag(258, starters[i])
            eng.close()
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for i in range(2):
        assert rel_err(out[i], ref[i]) < 1e-12
