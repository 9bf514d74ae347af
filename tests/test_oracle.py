"""Pin the oracle (the CPU restatement in oracle/) before it is trusted as the checker.

* reorder / SliceMap known answers of cppcore/tests/test_kpm.cpp:19-184;
* the reference's golden arrays of tests/test_kpm.py (LDOS, DOS, conductivity);
* FP64 moments of the reference's own NumPy KPM (``_PythonImpl``) on supplied starters.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from tests import models as TM


@pytest.fixture(scope="module")
def kat(oracle):
    m = TM.cpp_fixture_model()
    mn, mx, _ = oracle.lanczos(m.hamiltonian)
    a, b = oracle.scale(mn, mx)
    return m, a, b


def _sizes(oracle, r, M):
    return [oracle.slicemap_index(r["slices"], r["src_offset"], r["dest_offset"], n, M) for n in range(M)]


def test_reorder_kat_diagonal(oracle, kat):
    """cppcore/tests/test_kpm.cpp:34-96"""
    m, a, b = kat
    s = m.system
    n = s.num_sites
    i = s.find_nearest([0, 0.07], "B")
    r = oracle.optimize(m.hamiltonian, [i], [i], a, b)
    assert list(r["src"]) == [0] and list(r["dest"]) == [0]
    assert r["slices"][0] == 1 and r["slices"][-1] == n and r["slices"].size == 5
    assert (r["src_offset"], r["dest_offset"]) == (0, 0)
    assert _sizes(oracle, r, 6) == [0, 1, 2, 2, 1, 0]
    assert _sizes(oracle, r, 9) == [0, 1, 2, 3, 4, 3, 2, 1, 0]
    assert _sizes(oracle, r, 12) == [0, 1, 2, 3, 4, 4, 4, 4, 3, 2, 1, 0]

    i1, i2 = s.find_nearest([0, -0.07], "A"), s.find_nearest([0, 0.07], "B")
    assert i1 != i2
    r = oracle.optimize(m.hamiltonian, [i1, i2], [i1, i2], a, b)
    assert list(r["src"]) == [0, 3] and list(r["dest"]) == [0, 3]
    assert r["slices"].size == 5 and (r["src_offset"], r["dest_offset"]) == (1, 1)
    assert _sizes(oracle, r, 6) == [1, 2, 3, 3, 2, 1]
    assert _sizes(oracle, r, 9) == [1, 2, 3, 4, 4, 4, 3, 2, 1]
    assert _sizes(oracle, r, 12) == [1, 2, 3, 4, 4, 4, 4, 4, 4, 3, 2, 1]

    idx = [s.find_nearest([0, 0.07], "B"), s.find_nearest([0, -0.07], "A"), s.find_nearest([0, 0.35], "A")]
    r = oracle.optimize(m.hamiltonian, idx, idx, a, b)
    assert list(r["src"]) == [0, 1, 15] and list(r["dest"]) == [0, 1, 15]
    assert r["slices"].size == 5 and (r["src_offset"], r["dest_offset"]) == (3, 3)
    assert _sizes(oracle, r, 6) == [3, 4, 4, 4, 4, 3]
    assert _sizes(oracle, r, 9) == [3, 4, 4, 4, 4, 4, 4, 4, 3]
    assert _sizes(oracle, r, 12) == [3, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 3]


def test_reorder_kat_offdiagonal(oracle, kat):
    """cppcore/tests/test_kpm.cpp:98-171"""
    m, a, b = kat
    s = m.system
    i, j = s.find_nearest([0, 0.35], "A"), s.find_nearest([0, 0.07], "B")
    r = oracle.optimize(m.hamiltonian, [i], [j], a, b)
    assert list(r["src"]) == [0] and list(r["dest"]) == [8]
    assert r["slices"][0] == 1 and r["slices"][-1] == s.num_sites and r["slices"].size == 8
    assert (r["src_offset"], r["dest_offset"]) == (0, 3)
    assert _sizes(oracle, r, 6) == [0, 1, 2, 3, 4, 3]
    assert _sizes(oracle, r, 9) == [0, 1, 2, 3, 4, 5, 5, 4, 3]
    assert _sizes(oracle, r, 12) == [0, 1, 2, 3, 4, 5, 6, 7, 6, 5, 4, 3]
    assert _sizes(oracle, r, 14) == [0, 1, 2, 3, 4, 5, 6, 7, 7, 7, 6, 5, 4, 3]

    js = [s.find_nearest([0, 0.07], "B"), s.find_nearest([0.12, 0.14], "A"), s.find_nearest([0.12, 0.28], "B")]
    r = oracle.optimize(m.hamiltonian, [i], js, a, b)
    assert list(r["src"]) == [0] and list(r["dest"]) == [8, 5, 2]
    assert r["slices"].size == 8 and (r["src_offset"], r["dest_offset"]) == (0, 3)

    i1, i2 = s.find_nearest([0, 0.35], "A"), s.find_nearest([0, -0.35], "B")
    j1, j2 = s.find_nearest([0.12, 0.28], "B"), s.find_nearest([-0.12, 0.28], "B")
    r = oracle.optimize(m.hamiltonian, [i1, i2], [j1, j2], a, b)
    assert list(r["src"]) == [0, 18] and list(r["dest"]) == [2, 1]
    assert r["slices"].size == 8 and (r["src_offset"], r["dest_offset"]) == (7, 1)
    assert _sizes(oracle, r, 6) == [6, 5, 4, 3, 2, 1]
    assert _sizes(oracle, r, 9) == [7, 7, 7, 6, 5, 4, 3, 2, 1]
    assert _sizes(oracle, r, 12) == [7, 7, 7, 7, 7, 7, 6, 5, 4, 3, 2, 1]


def test_scaling_inserts_diagonal(oracle):
    """cppcore/tests/test_kpm.cpp:174-184: b != 0 adds a full diagonal"""
    m = TM.cpp_fixture_model_plain()
    a, b = oracle.scale(-12, 10)
    assert b != 0
    r = oracle.optimize(m.hamiltonian, [0], [0], a, b)
    assert r["h2"].nnz == m.hamiltonian.nnz + m.hamiltonian.shape[0]


def test_scale_rounds_small_b_to_zero(oracle):
    a, b = oracle.scale(-8.0, 8.0001)
    assert b == 0.0
    a, b = oracle.scale(-1.0, 3.0)
    assert a == pytest.approx(2.0 * 1.01, rel=1e-7) and b == 1.0


def test_kernels_and_rounding(oracle):
    """kpm/Kernel.hpp:9-13, Kernel.cpp:6-50"""
    assert [oracle.round_num_moments(n) for n in (0, 2, 3, 6, 7, 2049)] == [2, 2, 6, 6, 10, 2050]
    g = oracle.damping("jackson", 4.0, 10)
    assert g[0] == pytest.approx(1.0) and np.all(np.diff(g) < 0)
    gl = oracle.damping("lorentz", 4.0, 10)
    assert gl[0] == pytest.approx(1.0) and gl[-1] == pytest.approx(np.sinh(0.4) / np.sinh(4.0))
    assert np.all(oracle.damping("dirichlet", 4.0, 7) == 1.0)


@pytest.mark.parametrize("name", list(TM.LDOS_MODELS))
def test_golden_ldos(oracle, baselines, name):
    """tests/test_kpm.py:25-47 (Lorentz kernel, 4 configurations, rtol 1e-3)"""
    kind, size = TM.LDOS_MODELS[name]
    m = TM.graphene(kind, size)
    energy = np.linspace(0, 2, 25)
    idx = m.system.find_nearest([0, 0.07])
    expected = baselines["ldos[%s]" % name]
    for cfg in [dict(matrix_format="CSR", optimal_size=False, interleaved=False),
                dict(matrix_format="CSR", optimal_size=True, interleaved=False),
                dict(matrix_format="CSR", optimal_size=False, interleaved=True),
                dict(matrix_format="ELL", optimal_size=True, interleaved=True)]:
        r = oracle.core_ldos(m.hamiltonian, [idx], energy, 0.15, kernel="lorentz", **cfg)[:, 0]
        np.testing.assert_allclose(r, expected, rtol=1e-3, atol=1e-6)


@pytest.mark.parametrize("name", list(TM.DOS_MODELS))
def test_golden_dos(oracle, baselines, name):
    """tests/test_kpm.py:146-165: pins the default-seed mt19937 starter and the site order"""
    kind, size = TM.DOS_MODELS[name]
    m = TM.graphene(kind, size)
    energy = np.linspace(0, 2, 25)
    for cfg in [dict(optimal_size=False, interleaved=False), dict(optimal_size=True, interleaved=True)]:
        r, _ = oracle.core_dos(m.hamiltonian, energy, 0.15, 1, kernel="lorentz", matrix_format="ELL", **cfg)
        np.testing.assert_allclose(r, baselines["dos[%s]" % name], rtol=1e-3, atol=1e-6)


def test_golden_ldos_mos2(oracle, baselines):
    """tests/test_kpm.py:22-47, the multi-orbital case: the three-band MoS2 model
    (group6_tmd.monolayer_3band, restated by lattice.build_tmd_3band) in a 6 nm rectangle, LDOS of
    the three orbitals of the site nearest (0, 0.07) without reduction (rtol 1e-3, atol 1e-6)."""
    from pybinding_gb300 import lattice as L
    m = L.build_tmd_3band(L.rectangle(6), "MoS2")
    assert m.is_multiorbital and m.hamiltonian.shape == (3 * m.system.num_sites,) * 2
    idx = m.system.to_hamiltonian_indices(m.system.find_nearest([0, 0.07]))
    assert idx.size == 3
    energy = np.linspace(0, 2, 25)
    for cfg in [dict(matrix_format="CSR", optimal_size=False, interleaved=False),
                dict(matrix_format="CSR", optimal_size=True, interleaved=False),
                dict(matrix_format="CSR", optimal_size=False, interleaved=True),
                dict(matrix_format="ELL", optimal_size=True, interleaved=True)]:
        r = oracle.core_ldos(m.hamiltonian, idx, energy, 0.15, kernel="lorentz", **cfg)
        np.testing.assert_allclose(r, baselines["ldos[mos2]"], rtol=1e-3, atol=1e-6)


@pytest.mark.parametrize("name", list(TM.COND_MODELS))
def test_golden_conductivity(oracle, baselines, name):
    """tests/test_kpm.py:176-197 (rtol 1e-2, atol 1e-5)"""
    kind, size = TM.COND_MODELS[name]
    m = TM.graphene(kind, size)
    x = m.system.x
    r = oracle.core_conductivity(m.hamiltonian, x, x, np.linspace(-2, 2, 25), 0.5, 0.0, 1, 200,
                                 energy_range=(-9, 9), kernel="lorentz", matrix_format="ELL",
                                 optimal_size=False, interleaved=False).real
    np.testing.assert_allclose(r, baselines["conductivity[%s]" % name], rtol=1e-2, atol=1e-5)


@pytest.mark.parametrize("tag", ["c128", "f64"])
def test_python_impl_moments(oracle, python_impl, tag):
    """The oracle's FP64 recursion equals the reference's _PythonImpl on the same starters."""
    d = python_impl
    n = d[tag + "_indptr"].size - 1
    h = sp.csr_matrix((d[tag + "_data"], d[tag + "_indices"], d[tag + "_indptr"]), shape=(n, n))
    a, b = d[tag + "_ab"]
    ref = d[tag + "_moments"]
    M = ref.shape[1]
    r = oracle.optimize(h, [0], [0], a, b)
    starters = oracle.reorder_vector(d[tag + "_starters"], r["reorder_map"])
    for ell in (False, True):
        for interleaved in (False, True):
            if interleaved and (M - 2) % 4:
                continue
            got = oracle.moments_diag(r["h2"], starters, M, slices=r["slices"], ell=ell, interleaved=interleaved)
            err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
            assert err < 1e-12, (ell, interleaved, err)


def test_starters_are_reference_mt19937(oracle):
    """Starter.cpp:59-81 with std::mt19937 default seed 5489: first draws are fixed."""
    r = oracle.random_starters(5, 2, np.float32)
    # uniform floats of the default mt19937: 0.8147, 0.1355, 0.9058, 0.8350, 0.1270, ...
    assert list(r[0]) == [1, -1, 1, 1, -1]
    c = oracle.random_starters(3, 1, np.complex128)
    assert np.allclose(np.abs(c), 1.0)


def test_lanczos_matches_exact_extremes(oracle):
    """compute/lanczos.hpp:101-154: bounds within the 0.002% convergence target."""
    m = TM.graphene("const_potential", 4)
    h = m.hamiltonian.astype(np.float64)
    mn, mx, loops = oracle.lanczos(h)
    ev = np.linalg.eigvalsh(h.toarray())
    assert mn == pytest.approx(ev[0], rel=1e-3) and mx == pytest.approx(ev[-1], rel=1e-3)
    assert 0 < loops < 1000
