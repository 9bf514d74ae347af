"""The builders of KPM inputs against the reference's system baselines and each other.

The host build (``pybinding_gb300.lattice``, numpy) restates pybinding's foundation,
polygon, dangling-site and Hamiltonian code; it is pinned bit for bit by the reference's
own system baselines (pickled ``System`` objects of its shape and system tests) and, via
the site order, by its DOS golden arrays. The GPU build (include/kpm_lattice.h) must give
the same model bit for bit: positions, sublattice ranges, CSR structure and values.
"""
import math

import numpy as np
import pytest

from pybinding_gb300 import _native, lattice as L


def assert_same_model(got, ref):
    hg, hr = got.hamiltonian, ref.hamiltonian
    assert hg.shape == hr.shape
    assert hg.dtype == hr.dtype
    np.testing.assert_array_equal(hg.indptr, hr.indptr)
    np.testing.assert_array_equal(hg.indices, hr.indices)
    # bitwise: compare the raw bytes (signed zeros and NaNs included)
    assert hg.data.tobytes() == hr.data.tobytes()
    for a, b in zip(got.system.positions, ref.system.positions):
        assert a.dtype == b.dtype == np.float32
        assert a.tobytes() == b.tobytes()
    assert got.system.sub_ranges == ref.system.sub_ranges


# ---------------------------------------------------------------- the reference's system baselines
# nearest-neighbour graphene cut by the shapes of tests/test_shape.py:8-14 and the hexagon
# of tests/test_system.py:8 (positions, site counts per sublattice, hopping pairs)
SYSTEM_SHAPES = {
    "polygon_expected[triangle]": lambda: (L.regular_polygon(3, 1.1), (0.0, 0.0)),
    "polygon_expected[triangle90]": lambda: (L.regular_polygon(3, 1.1, math.pi / 2), (0.0, 0.0)),
    "polygon_expected[diamond]": lambda: (L.regular_polygon(4, 1.0), (0.0, 0.0)),
    "polygon_expected[square]": lambda: (L.regular_polygon(4, 1.0, math.pi / 4), (0.0, 0.0)),
    "polygon_expected[pentagon]": lambda: (L.regular_polygon(5, 1.0), (0.0, 0.0)),
    "expected[graphene-monolayer]": lambda: L.hexagon_ac(1.0),
}


@pytest.fixture(scope="module")
def system_baselines():
    import os
    from tests.conftest import GOLDEN
    return dict(np.load(os.path.join(GOLDEN, "system_baselines.npz")))


def assert_matches_system_baseline(model, base, case):
    x, y, z = model.system.positions
    assert x.tobytes() == base[case + "/x"].tobytes()  # bit for bit, float32
    assert y.tobytes() == base[case + "/y"].tobytes()
    assert z.tobytes() == base[case + "/z"].tobytes()
    counts = base[case + "/site_counts"]
    assert model.system.sub_ranges == {"A": (0, int(counts[0])), "B": (int(counts[0]), int(counts.sum()))}
    h = model.hamiltonian.tocoo()
    upper = h.row < h.col
    rows, cols = base[case + "/hop_rows"], base[case + "/hop_cols"]
    mine = sorted(zip(h.row[upper].tolist(), h.col[upper].tolist()))
    ref = sorted(zip(np.minimum(rows, cols).tolist(), np.maximum(rows, cols).tolist()))
    assert mine == ref
    np.testing.assert_array_equal(h.data[upper], np.float32(L.GRAPHENE_T))


@pytest.mark.parametrize("case", sorted(SYSTEM_SHAPES))
def test_host_build_matches_reference_system_baseline(system_baselines, case):
    v, offset = SYSTEM_SHAPES[case]()
    assert_matches_system_baseline(L.build_honeycomb(v, lattice_offset=offset), system_baselines, case)


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(SYSTEM_SHAPES))
def test_gpu_build_matches_reference_system_baseline(system_baselines, case):
    v, offset = SYSTEM_SHAPES[case]()
    assert_matches_system_baseline(L.build_honeycomb(v, lattice_offset=offset, device="gpu"), system_baselines, case)


# ---------------------------------------------------------------- host-side checks (no GPU)

def test_builder_rejects_bad_arguments_before_touching_the_gpu():
    with pytest.raises(ValueError, match="L must be >= 3"):
        _native.LatticeBuild.cubic(2)
    with pytest.raises(ValueError, match="foundation size"):
        _native.LatticeBuild.honeycomb(0, 4, np.zeros(3), np.ones(3), np.ones(3), np.zeros((2, 3)),
                                       L._HONEYCOMB_HOPS, L.rectangle(1.0), 2)
    with pytest.raises(ValueError, match="min_neighbors"):
        _native.LatticeBuild.honeycomb(4, 4, np.zeros(3), np.ones(3), np.ones(3), np.zeros((2, 3)),
                                       L._HONEYCOMB_HOPS, L.rectangle(1.0), -1)
    with pytest.raises(ValueError, match="device must be"):
        L.build_honeycomb(L.rectangle(1.0), device="cpu")


# ---------------------------------------------------------------- device build (GPU)

def _hexagon(r):
    ang = np.arange(6) * math.pi / 3
    return np.stack([r * np.cos(ang), r * np.sin(ang)], axis=1).astype(np.float32)


def _triangle(s):
    # one horizontal edge: exercises the skipped (equal-y) edges of the ray casting
    return np.array([[-s / 2, -s / 3], [s / 2, -s / 3], [0, 2 * s / 3]], np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("num_sites", [300, 3000, 40000])
def test_graphene_flake_matches_host_build(num_sites):
    assert_same_model(L.graphene_flake(num_sites, device="gpu"), L.graphene_flake(num_sites))


@pytest.mark.gpu
@pytest.mark.parametrize("shape", ["hexagon", "triangle", "rectangle_tilted"])
def test_polygons_match_host_build(shape):
    if shape == "hexagon":
        v = _hexagon(4.0)
    elif shape == "triangle":
        v = _triangle(9.0)
    else:
        c, s = math.cos(0.3), math.sin(0.3)
        v = (L.rectangle(6.0, 3.5).astype(np.float64) @ np.array([[c, s], [-s, c]])).astype(np.float32)
    for mn in (1, 2, 3):
        assert_same_model(L.build_honeycomb(v, min_neighbors=mn, device="gpu"), L.build_honeycomb(v, min_neighbors=mn))


@pytest.mark.gpu
def test_test_fixture_lattice_matches_host_build():
    """float32 lattice constants and min_neighbors = 1 (the C++ test fixture)."""
    kw = dict(min_neighbors=1, float_constants=True)
    assert_same_model(L.build_honeycomb(L.rectangle(0.6, 0.8), device="gpu", **kw),
                      L.build_honeycomb(L.rectangle(0.6, 0.8), **kw))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["potential_f32", "anderson_f64", "field_c64", "field_c128", "strain_f64",
                                  "mass_c64"])
def test_modifiers_match_host_build(case):
    kw = {
        "potential_f32": dict(onsite_modifiers=[L.constant_potential(0.5)]),
        "anderson_f64": dict(onsite_modifiers=[L.anderson_disorder(1.0, 3)], is_double=True),
        "field_c64": dict(hopping_modifiers=[L.constant_magnetic_field(200.0)], is_complex=True),
        "field_c128": dict(hopping_modifiers=[L.constant_magnetic_field(200.0)], is_complex=True, is_double=True,
                           onsite_modifiers=[L.anderson_disorder(0.3, 5)]),
        "strain_f64": dict(hopping_modifiers=[L.strained_hopping(L.sinusoidal_strain(0.05, 20.0))], is_double=True),
        "mass_c64": dict(onsite_modifiers=[L.mass_term(0.1)], is_complex=True),
    }[case]
    assert_same_model(L.graphene_flake(5000, device="gpu", **kw), L.graphene_flake(5000, **kw))


@pytest.mark.gpu
def test_empty_polygon_gives_an_empty_model():
    v = np.array([[0.01, 0.01], [0.02, 0.01], [0.02, 0.02]], np.float32)
    got = L.build_honeycomb(v, device="gpu")
    ref = L.build_honeycomb(v)
    assert got.hamiltonian.shape == ref.hamiltonian.shape == (0, 0)
    assert_same_model(got, ref)


@pytest.mark.gpu
def test_hopping_list_is_in_host_order():
    v = L.rectangle(3.0, 2.0)
    b = _native.LatticeBuild.honeycomb(*_frame_args(v), min_neighbors=2)
    rows, cols = b.hoppings()
    n, n0, nh, max_nnz = b.sizes()
    b.close()
    ref = L.build_honeycomb(v)
    h = ref.hamiltonian.tocoo()
    upper = h.row < h.col
    assert nh == int(upper.sum()) and max_nnz == 2 * nh + n
    assert np.all(rows < n0) and np.all(cols >= n0)
    # the same set of bonds; within each direction rows ascend
    assert set(zip(rows.tolist(), cols.tolist())) == set(zip(h.row[upper].tolist(), h.col[upper].tolist()))


def _frame_args(v):
    v0, v1, sub_pos, origin, s0, s1 = L._honeycomb_frame(v, L.GRAPHENE_A, L.GRAPHENE_A_CC, False)
    return s0, s1, origin, v0, v1, sub_pos, L._HONEYCOMB_HOPS, v


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex64, np.complex128])
@pytest.mark.parametrize("size", [3, 5, 17])
def test_cubic_matches_host_build(dtype, size):
    rng = np.random.default_rng(size)
    onsite = rng.uniform(-8.25, 8.25, size ** 3)
    onsite[::7] = 0.0  # zeros are not stored
    assert_same_model(L.simple_cubic_periodic(size, onsite=onsite, dtype=dtype, device="gpu"),
                      L.simple_cubic_periodic(size, onsite=onsite, dtype=dtype))
    assert_same_model(L.simple_cubic_periodic(size, dtype=dtype, device="gpu"),
                      L.simple_cubic_periodic(size, dtype=dtype))


@pytest.mark.gpu
def test_large_flake_matches_host_build():
    """A 1M-site disordered flake: foundation of ~2M sites, several scan tiles per array."""
    kw = dict(onsite_modifiers=[L.anderson_disorder(1.0, 11)])
    assert_same_model(L.graphene_flake(1_000_000, device="gpu", **kw), L.graphene_flake(1_000_000, **kw))


@pytest.mark.gpu
def test_gpu_built_model_runs_the_same_kpm():
    from pybinding_gb300 import kpm
    ref = L.graphene_flake(4000, onsite_modifiers=[L.anderson_disorder(1.0, 2)])
    got = L.graphene_flake(4000, onsite_modifiers=[L.anderson_disorder(1.0, 2)], device="gpu")
    assert_same_model(got, ref)
    e = np.linspace(-8, 8, 41)
    # the blocks add their moment partials with FP64 atomics in no fixed order
    np.testing.assert_allclose(kpm(got).calc_dos(e, 0.1, num_random=2).data,
                               kpm(ref).calc_dos(e, 0.1, num_random=2).data, rtol=1e-9)


def _mass_hexagon():
    v, offset = L.hexagon_ac(10)
    return L.build_honeycomb(v, onsite_modifiers=[L.mass_term(1)], lattice_offset=offset)


def test_mass_term_ldos_is_sublattice_antisymmetric_in_the_oracle(oracle):
    """The inputs of the reference's test_ldos_sublattice (tests/test_kpm.py:117-123): with a
    mass term the A and B LDOS at the centre mirror each other in energy (oracle, CPU)."""
    m = _mass_hexagon()
    e = np.linspace(-5, 5, 50)
    a, b = (oracle.core_ldos(m.hamiltonian, [m.system.find_nearest([0, 0], sub)], e, 0.1)[:, 0] for sub in "AB")
    np.testing.assert_allclose(a, b[::-1], rtol=1e-3, atol=1e-6)


@pytest.mark.gpu
def test_ldos_sublattice():
    """tests/test_kpm.py:117-123 of the reference through the pb.kpm-compatible API."""
    from pybinding_gb300 import kpm
    k = kpm(_mass_hexagon(), silent=True)
    a, b = (k.calc_ldos(np.linspace(-5, 5, 50), 0.1, [0, 0], sub) for sub in ("A", "B"))
    np.testing.assert_allclose(a.data, b.data[::-1], rtol=1e-3, atol=1e-6)


@pytest.mark.gpu
def test_kpm_reuse():
    """tests/test_kpm.py:104-114 of the reference: one KPM object used for several
    calculations gives what fresh objects give."""
    from pybinding_gb300 import kpm
    v, offset = L.hexagon_ac(10)
    model = L.build_honeycomb(v, lattice_offset=offset)
    k = kpm(model, silent=True)
    energy = np.linspace(-5, 5, 50)
    for position in [0, 0], [6, 0]:
        actual = k.calc_ldos(energy, 0.1, position)
        expected = kpm(model).calc_ldos(energy, 0.1, position)
        np.testing.assert_allclose(actual.data, expected.data, rtol=1e-3, atol=1e-6)
