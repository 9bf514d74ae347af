"""Parameter sweeps (``pybinding/parallel.py``): factories, batching of deferred LDOS jobs
into ragged GPU batches, and the sweep results."""
import numpy as np
import pytest

import pybinding_gb300 as pbg
from pybinding_gb300 import lattice as L, parallel
from pybinding_gb300.chebyshev import Deferred


def test_parallelize_makes_the_product_of_the_variables():
    @pbg.parallelize(a=[1, 2, 3], b=[10, 20])
    def factory(a, b, energy=np.linspace(0, 1, 4), scale=2.0):
        return Deferred(lambda: np.full(4, scale * (a + b)))

    assert factory.sequence == [(1, 10), (1, 20), (2, 10), (2, 20), (3, 10), (3, 20)]
    assert set(factory.fixtures) == {"energy", "scale"}
    data = pbg.parallel_for(factory)
    assert [float(d[0]) for d in data] == [22.0, 42.0, 24.0, 44.0, 26.0, 46.0]
    nd = pbg.ndsweep(factory, labels=dict(axes=["a", "b", "E"]))
    assert nd.data.shape == (3, 2, 4) and nd.labels["x"] == "a"
    np.testing.assert_array_equal(nd.data[2, 1], np.full(4, 46.0))


def test_sweep_stacks_one_row_per_value():
    @pbg.parallelize(x=np.linspace(0, 1, 5))
    def factory(x, energy=np.linspace(-1, 1, 7)):
        return Deferred(lambda: (x * energy)[:, None])

    s = pbg.sweep(factory, labels=dict(x="x", y="E"))
    assert s.data.shape == (5, 7)
    np.testing.assert_allclose(s.data[4], np.linspace(-1, 1, 7))
    assert s.labels["y"] == "E" and s.labels["title"] == ""


def _flake(n, seed, double=False):
    return L.graphene_flake(n, onsite_modifiers=[L.anderson_disorder(0.5, seed)], is_double=double)


def test_deferred_ldos_jobs_are_grouped_into_batches(monkeypatch):
    """Jobs with equal settings and scalar type share a batch, split at MAX_BATCH_ROWS;
    other jobs run alone, in order. (The batch runner is replaced: no GPU here.)"""
    runs = []

    def fake_batch(chunk):
        runs.append([d.impl.model.hamiltonian.shape[0] for d, _ in chunk])
        for d, site in chunk:
            assert site == d.site
            d.result = np.full((3, 1), float(site))

    monkeypatch.setattr(parallel, "_run_ldos_batch", fake_batch)
    e = np.linspace(-1, 1, 3)
    f32 = [_flake(n, i) for i, n in enumerate((300, 500, 400))]
    f64 = [_flake(n, 9 + i, double=True) for i, n in enumerate((350, 450))]
    jobs = [pbg.kpm(m).deferred_ldos(e, 0.1, [0, 0]) for m in f32 + f64]
    other = Deferred(lambda: "plain")
    parallel.compute_all(jobs[:2] + [other] + jobs[2:])
    assert runs == [[f32[0].hamiltonian.shape[0], f32[1].hamiltonian.shape[0], f32[2].hamiltonian.shape[0]],
                    [f64[0].hamiltonian.shape[0], f64[1].hamiltonian.shape[0]]]
    assert other.result == "plain"
    assert all(j.result is not None for j in jobs)
    # a row cap splits a group into several batches
    runs.clear()
    four = [_flake(n, 30 + i) for i, n in enumerate((500, 500, 300, 300))]
    rows = [m.hamiltonian.shape[0] for m in four]
    monkeypatch.setattr(parallel, "MAX_BATCH_ROWS", rows[0] + rows[1])
    parallel.compute_all([pbg.kpm(m).deferred_ldos(e, 0.1, [0, 0]) for m in four])
    assert runs == [rows[:2], rows[2:]]
    # a different broadening is another group
    runs.clear()
    monkeypatch.setattr(parallel, "MAX_BATCH_ROWS", 1 << 26)
    jobs = [pbg.kpm(m).deferred_ldos(e, b, [0, 0]) for m in f32 for b in (0.1, 0.2)]
    parallel.compute_all(jobs)
    assert sorted(len(r) for r in runs) == [3, 3]


@pytest.mark.gpu
@pytest.mark.parametrize("double", [True, False])
def test_batched_ldos_matches_single_model_ldos(double):
    models = [_flake(n, 20 + i, double) for i, n in enumerate((3000, 1800, 5200, 900))]
    e = np.linspace(-8, 8, 61)
    batch = pbg.kpm_batch(models)
    got = batch.calc_ldos(e, 0.1, position=[0.1, 0.2])
    batch.close()
    tol = 1e-9 if double else 2e-5
    for m, g in zip(models, got):
        ref = pbg.kpm(m).calc_ldos(e, 0.1, [0.1, 0.2]).data
        err = np.max(np.abs(g.data - ref)) / np.max(np.abs(ref))
        print("batched vs single LDOS (%s): %.2e" % ("f64" if double else "f32", err))
        assert err < tol


@pytest.mark.gpu
def test_sweep_of_deferred_ldos_runs_as_one_batch(monkeypatch):
    energy = np.linspace(-3, 3, 41)
    strengths = [0.0, 0.5, 1.0, 2.0, 3.0]
    batches = []
    real = parallel._run_ldos_batch

    def spy(chunk):
        batches.append(len(chunk))
        real(chunk)

    monkeypatch.setattr(parallel, "_run_ldos_batch", spy)

    @pbg.parallelize(w=strengths)
    def factory(w, energy=energy, broadening=0.15):
        model = L.graphene_flake(2500, onsite_modifiers=[L.anderson_disorder(w, 3)], is_double=True)
        return pbg.kpm(model).deferred_ldos(energy, broadening, position=[0, 0])

    s = pbg.sweep(factory)
    assert batches == [len(strengths)]
    assert s.data.shape == (len(strengths), energy.size)
    for w, row in zip(strengths, s.data):
        model = L.graphene_flake(2500, onsite_modifiers=[L.anderson_disorder(w, 3)], is_double=True)
        ref = pbg.kpm(model).calc_ldos(energy, 0.15, [0, 0]).data
        assert np.max(np.abs(row - ref)) / np.max(np.abs(ref)) < 1e-9


def test_batch_engine_from_engines_checks_its_members():
    from pybinding_gb300 import _binding
    a = _binding.Engine(_flake(300, 1).hamiltonian)
    b = _binding.Engine(_flake(400, 2, double=True).hamiltonian)
    with pytest.raises(ValueError, match="share the scalar type"):
        _binding.engine_batch([a, b])
    two = pbg.kpm_batch([_flake(300, 3), _flake(200, 4)]).engine
    with pytest.raises(ValueError, match="one system each"):
        _binding.engine_batch([a, two])
    c = _binding.Engine(_flake(500, 5).hamiltonian)
    batch = _binding.engine_batch([a, c])
    assert batch.num_systems == 2 and batch.rows == a.rows + c.rows
    np.testing.assert_array_equal(batch.system_offsets, [0, a.rows, a.rows + c.rows])
    batch.close()


@pytest.mark.gpu
def test_batch_engine_from_engines_matches_block_diagonal_batch():
    from pybinding_gb300 import _binding
    models = [_flake(n, 40 + i, double=True) for i, n in enumerate((2000, 3100, 700))]
    members = [_binding.Engine(m.hamiltonian) for m in models]
    members[1].scaling_factors()  # bounds found by a member are kept by the batch
    joined = _binding.engine_batch(members)
    ref = pbg.kpm_batch(models).engine
    e = np.linspace(-8, 8, 51)
    for s in range(3):
        assert joined.scaling_factors(s) == ref.scaling_factors(s)
    np.testing.assert_allclose(joined.calc_dos(e, 0.1, 2), ref.calc_dos(e, 0.1, 2), rtol=1e-12, atol=0)
    np.testing.assert_allclose(joined.calc_ldos_batch([5, 7, 9], e, 0.1), ref.calc_ldos_batch([5, 7, 9], e, 0.1),
                               rtol=1e-12, atol=0)


def test_batched_ldos_checks_its_sites_before_the_gpu():
    batch = pbg.kpm_batch([_flake(300, 1), _flake(200, 2)])
    with pytest.raises(ValueError, match="one LDOS site per system"):
        batch.engine.calc_ldos_batch([0], np.linspace(-1, 1, 5), 0.1)
    with pytest.raises(RuntimeError, match="LDOS index out of range"):
        batch.engine.calc_ldos_batch([0, 10 ** 6], np.linspace(-1, 1, 5), 0.1)
    batch.close()


# the reference's sweep tests (tests/test_parallel.py:14-50): deferred KPM LDOS of graphene
# hexagons (hexagon_ac(15), 22,686 sites) under constant potentials, Lorentz kernel,
# broadening 0.15 eV, energies linspace(0, 0.1, 10); compared as the reference does
# (rtol 1e-3, atol 1e-6)
def _sweep_baselines():
    import os
    from tests.conftest import GOLDEN
    folder = os.path.join(GOLDEN, "pbz_sweeps")
    return pbg.load(os.path.join(folder, "sweep.pbz")), pbg.load(os.path.join(folder, "ndsweep.pbz"))


def _hexagon_model(*potentials):
    v, offset = L.hexagon_ac(15)
    return L.build_honeycomb(v, onsite_modifiers=[L.constant_potential(p) for p in potentials], lattice_offset=offset)


def test_oracle_reproduces_the_reference_sweep_baselines(oracle):
    """The inputs of the reference's sweeps (hexagon_ac with its lattice offset, the potentials,
    the nearest site of sublattice B) through the oracle's Core::ldos match its baselines."""
    sweep, ndsweep = _sweep_baselines()
    energy = np.linspace(0, 0.1, 10)
    for i, v in enumerate(np.linspace(0, 0.1, 10)):
        m = _hexagon_model(v)
        ldos = oracle.core_ldos(m.hamiltonian, [m.system.find_nearest([0, 0], "B")], energy, 0.15, kernel="lorentz")
        np.testing.assert_allclose(ldos[:, 0], sweep.data[i], rtol=1e-3, atol=1e-6)
    v1s, v2s, _ = ndsweep.variables
    for i, j in ((0, 0), (4, 3), (1, 2)):
        m = _hexagon_model(v1s[i], v2s[j])
        ldos = oracle.core_ldos(m.hamiltonian, [m.system.find_nearest([0, 0])], energy, 0.15, kernel="lorentz")
        np.testing.assert_allclose(ldos[:, 0], ndsweep.data[i, j], rtol=1e-3, atol=1e-6)


@pytest.mark.gpu
def test_sweep_matches_the_reference_sweep_baseline():
    expected, _ = _sweep_baselines()

    @pbg.parallelize(v=np.linspace(0, 0.1, 10))
    def factory(v, energy=np.linspace(0, 0.1, 10)):
        kpm = pbg.kpm(_hexagon_model(v), kernel=pbg.lorentz_kernel())
        return kpm.deferred_ldos(energy, broadening=0.15, position=[0, 0], sublattice="B")

    labels = dict(title="test sweep", x="V (eV)", y="E (eV)", data="LDOS")
    result = pbg.sweep(factory, labels=labels)
    np.testing.assert_allclose(result.x, expected.x)
    np.testing.assert_allclose(result.y, expected.y)
    np.testing.assert_allclose(result.data, expected.data, rtol=1e-3, atol=1e-6)
    assert result.labels == expected.labels


@pytest.mark.gpu
def test_ndsweep_matches_the_reference_ndsweep_baseline():
    _, expected = _sweep_baselines()

    @pbg.parallelize(v1=np.linspace(0, 0.1, 5), v2=np.linspace(-0.2, 0.2, 4))
    def factory(v1, v2, energy=np.linspace(0, 0.1, 10)):
        kpm = pbg.kpm(_hexagon_model(v1, v2), kernel=pbg.lorentz_kernel())
        return kpm.deferred_ldos(energy, broadening=0.15, position=[0, 0])

    result = pbg.ndsweep(factory)
    assert result.data.shape == expected.data.shape
    np.testing.assert_allclose(result.data, expected.data, rtol=1e-3, atol=1e-6)
