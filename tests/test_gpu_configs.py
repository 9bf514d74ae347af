"""GPU parity at the sizes of the benchmark configurations, spatial LDOS, and Lanczos bounds.

Error measure for moments: max |mu - mu_ref| / max |mu_ref| over every vector and moment.
Tolerances: FP64 recursion <= 1e-10; FP32 recursion vectors with FP64 moment sums <= 1e-6
(the precision target of the FP32 form); functions of energy as for the moments.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from pybinding_gb300 import _native, kpm, kpm_batch, lattice as L

pytestmark = pytest.mark.gpu


# The reference (and the oracle) scale the spectral density by 2 / pi with a float pi, the
# quotient itself taken in float (numeric/constant.hpp:7, reconstruct.hpp:27), the engine in
# double: the two differ by this factor (engine / reference).
PI_RATIO = (2 / np.pi) / float(np.float32(2) / np.float32(np.pi))


def rel_err(got, ref):
    return float(np.max(np.abs(np.asarray(got) - np.asarray(ref))) / np.max(np.abs(ref)))


def _rademacher(n, count, seed):
    rng = np.random.default_rng(seed)
    return np.where(rng.integers(0, 2, size=(count, n)) == 0, -1.0, 1.0).astype(np.float32)


@pytest.mark.parametrize("precision,tol", [("fp32", 2e-6), ("fp32p", 2e-7), ("fp32x", 2e-7)])
def test_fp32_moments_of_a_full_size_flake(oracle, precision, tol):
    """One flake of the batched DOS workload at its largest size (400k sites, onsite disorder
    U[-0.5, 0.5] eV, float32 H), 64 Rademacher vectors, 4098 moments, Lanczos bounds: the FP32
    recursion (row sums of chained FMAs, compensated by one FMA per term, or by TwoSum and
    rounded once) against the FP64
    recursion of the same engine settings (bit-identical bounds) on every vector, and both
    against the FP64 oracle on two vectors with the engine's own (a, b)."""
    m = L.graphene_flake(400_000, onsite_modifiers=[L.anderson_disorder(1.0, 11)])
    h = m.hamiltonian.astype(np.float32)
    n = h.shape[0]
    st = _rademacher(n, 64, 5)
    M = 4096
    e32 = _native.Engine(h, _native.make_config(precision=precision))
    e64 = _native.Engine(h, _native.make_config(precision="fp64"))
    assert e32.energy_bounds() == e64.energy_bounds()  # deterministic Lanczos: the same bits
    a, b = e32.scaling_factors()
    m32 = e32.moments_diag(M, st[None])[0]
    m64 = e64.moments_diag(M, st[None])[0]
    e32.close()
    e64.close()
    assert m32.shape == (64, 4098)
    err = rel_err(m32, m64)
    print("full-size flake (%d sites), %s: vs FP64 per-vector %.3e, vector-averaged %.3e" % (
        n, precision, err, rel_err(m32.mean(0), m64.mean(0))))
    assert err <= tol
    r = oracle.optimize(h.astype(np.float64), [0], [0], a, b)
    ref = oracle.moments_diag(r["h2"], oracle.reorder_vector(st[:2].astype(np.float64), r["reorder_map"]), 4098,
                              slices=r["slices"])
    e64o = rel_err(m64[:2], ref)
    e32o = rel_err(m32[:2], ref)
    print("  vs FP64 oracle (2 vectors): FP64 %.3e, %s %.3e" % (e64o, precision, e32o))
    assert e64o <= 1e-10
    assert e32o <= tol


def test_dos_configuration_c128_60k_matches_oracle(oracle):
    """The 60k-site complex128 DOS configuration as configured: 60,074-site graphene flake
    (t = -2.8 eV, onsite 0), the reference's 8 random-phase starters (std::mt19937 default
    seed, e^{2 pi i u}), 2048 moments (2050 after rounding), Lanczos bounds. FP64 moments equal
    the oracle's on the engine's (a, b) to 1e-10, and the DOS on 1000 energies in [-9, 9] eV
    equals the oracle's reconstruction from those moments."""
    m = L.graphene_flake(60000, is_complex=True, is_double=True)
    h = m.hamiltonian.astype(np.complex128)
    n = h.shape[0]
    assert n == 60074
    eng = _native.Engine(h, _native.make_config())
    a, b = eng.scaling_factors()
    st = oracle.random_starters(n, 8, np.complex128)
    mu = eng.moments_diag(2048, st[None])[0]
    assert mu.shape == (8, 2050)
    r = oracle.optimize(h, [0], [0], a, b)
    ref = oracle.moments_diag(r["h2"], oracle.reorder_vector(st, r["reorder_map"]), 2050, slices=r["slices"])
    err = rel_err(mu, ref)
    print("c128 60k DOS moments vs oracle: %.3e" % err)
    assert err <= 1e-10
    # the DOS the engine reconstructs from its own starters (calc_dos draws the same starters)
    energy = np.linspace(-9, 9, 1000)
    broadening = 0.0125
    dos = eng.calc_dos(energy, broadening, 8)[0]
    M = eng.stats().num_moments
    mu_ref = oracle.moments_diag(r["h2"], oracle.reorder_vector(st, r["reorder_map"]), M, slices=r["slices"])
    mu_ref = mu_ref.mean(0).real * oracle.damping("jackson", 4.0, M)
    # reconstruct.hpp:16-45 in FP64 (the engine's reconstruction precision; pi in double)
    et = (energy - b) / a
    with np.errstate(invalid="ignore"):
        th = np.arccos(et)
        dref = 2 / (np.pi * a * np.sqrt(1 - et * et)) * (np.cos(np.outer(th, np.arange(M))) @ mu_ref)
    ok = np.isfinite(dref)
    assert np.array_equal(ok, np.isfinite(dos))  # |E~| >= 1 outside the bounds: NaN on both sides
    derr = rel_err(dos[ok], dref[ok])
    print("c128 60k DOS vs oracle reconstruction: %.3e" % derr)
    assert derr <= 1e-9
    eng.close()


def _periodic_graphene(nx, ny, t=-2.8, dtype=np.complex64):
    """Graphene on an nx x ny primitive-cell torus: sublattices A, B per cell, hoppings
    A(i,j)-B(i,j), A(i,j)-B(i-1,j+1), A(i,j)-B(i,j+1) (the three nearest neighbours of
    pybinding's graphene lattice) wrapped periodically."""
    cells = nx * ny
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    A = (i * ny + j).ravel()
    rows, cols = [], []
    for di, dj in ((0, 0), (-1, 1), (0, 1)):
        B = cells + (((i + di) % nx) * ny + (j + dj) % ny).ravel()
        rows += [A, B]
        cols += [B, A]
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    h = sp.csr_matrix((np.full(rows.size, t, dtype), (rows, cols)), shape=(2 * cells, 2 * cells))
    h.sum_duplicates()
    h.sort_indices()
    return h


def test_lanczos_reference_known_answer():
    """cppcore/tests/test_compute.cpp:8-25: periodic 5 x 5 graphene (complex64), precision
    1e-3 %: the bounds are +-3|t| and three runs take the same number of loops (here the
    bounds are the same bits too)."""
    h = _periodic_graphene(5, 5)
    runs = []
    for _ in range(3):
        eng = _native.Engine(h, _native.make_config(lanczos_precision=1e-3))
        runs.append(eng.energy_bounds())
        eng.close()
    mn, mx, loops = runs[0]
    expected = abs(3 * -2.8)
    eps = np.finfo(np.float32).eps * 100  # Catch's Approx default
    assert abs(mx - expected) <= eps * (1 + expected)
    assert abs(mn + expected) <= eps * (1 + expected)
    assert all(r == runs[0] for r in runs)
    print("Lanczos KAT: %.9f %.9f in %d loops" % (mn, mx, loops))


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.complex128])
def test_lanczos_bounds_match_oracle(oracle, dtype):
    """The engine's Lanczos (FP64 on the GPU, tridiagonal extremes by Sturm bisection) against the
    oracle's restatement of compute/lanczos.hpp:101-154 (H's scalar type, implicit QR) at the
    reference's default precision of 0.002 %. Double-precision H: the same algorithm in the
    same precision, so equal loop counts and bounds to 1e-12. float32 H: the reference works in
    float, the engine in double; the bounds then agree to the convergence precision (and the
    scaling factors a, b with them), and the largest difference is printed."""
    worst = 0.0
    for n_sites, seed in ((3000, 1), (20000, 2), (60000, 3)):
        m = L.graphene_flake(n_sites, onsite_modifiers=[L.anderson_disorder(1.0, seed)],
                             is_complex=np.iscomplexobj(np.zeros(1, dtype)))
        h = m.hamiltonian.astype(dtype)
        eng = _native.Engine(h, _native.make_config())
        mn, mx, loops = eng.energy_bounds()
        a, b = eng.scaling_factors()
        eng.close()
        omn, omx, oloops = oracle.lanczos(h, 0.002)
        oa, ob = oracle.scale(omn, omx)
        d = max(abs(mn - omn) / abs(omn), abs(mx - omx) / abs(omx))
        da = abs(a - oa) / oa
        worst = max(worst, d)
        print("%s %d sites: engine (%.9f, %.9f, %d loops), oracle (%.9f, %.9f, %d loops); rel diff bounds "
              "%.2e, a %.2e, b %.2e" % (np.dtype(dtype).name, h.shape[0], mn, mx, loops, omn, omx, oloops, d, da,
                                         abs(b - ob)))
        if dtype == np.float32:
            assert d <= 2e-5          # the convergence precision, 0.002 %
            assert abs(loops - oloops) <= 5
        else:
            assert d <= 1e-12
            assert loops == oloops
    print("largest relative bound difference (%s): %.2e" % (np.dtype(dtype).name, worst))


def _circle(cx, cy, r):
    return lambda x, y, z: (x - cx) ** 2 + (y - cy) ** 2 <= r * r


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-10), (np.float32, 1e-6)])
def test_spatial_ldos_matches_oracle(oracle, dtype, tol):
    """KPM.calc_spatial_ldos (KPM.cpp:67-94): the LDOS at every site inside a shape (and of one
    sublattice inside it) against the oracle's Core::ldos over the same Hamiltonian indices."""
    m = L.build_honeycomb(L.rectangle(12), onsite_modifiers=[L.anderson_disorder(0.4, 9)])
    m.hamiltonian = m.hamiltonian.astype(dtype)
    energy = np.linspace(-1.5, 1.5, 31)
    rng = (-9.5, 9.5)
    k = kpm(m, energy_range=rng)
    for sub in ("", "A", "B"):
        sl = k.calc_spatial_ldos(energy, 0.08, _circle(0.3, -0.2, 1.1), sublattice=sub)
        x, y, z = m.system.positions
        inside = _circle(0.3, -0.2, 1.1)(x, y, z)
        s0, s1 = m.system.sublattice_range(sub)
        idx = np.nonzero(inside & (np.arange(x.size) >= s0) & (np.arange(x.size) < s1))[0]
        assert np.array_equal(sl.indices, idx) and idx.size > 10
        ref = oracle.core_ldos(m.hamiltonian.astype(np.float64), idx, energy, 0.08, energy_range=rng)
        ref = ref * PI_RATIO
        assert sl.data.shape == ref.shape == (energy.size, idx.size)
        err = rel_err(sl.data, ref)
        print("spatial LDOS %s sublattice '%s' (%d sites): %.3e" % (np.dtype(dtype).name, sub, idx.size, err))
        assert err <= tol
        # the value at a site is the LDOS of that site (SpatialLDOS.ldos, chebyshev.py:33-49)
        j = idx.size // 2
        single = sl.ldos([x[idx[j]], y[idx[j]]])
        np.testing.assert_array_equal(single.data, sl.data[:, j])


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-10), (np.float32, 1e-6)])
def test_spatial_ldos_of_a_3d_anderson_cube_matches_oracle(oracle, dtype, tol):
    """The LDOS part of the 3D Anderson configuration on a small cube: 12^3 periodic simple cubic,
    t = -1, onsite U[-8.25, 8.25], LDOS at 64 sites (unit vectors batched as one block),
    against the oracle's Core::ldos."""
    Lc = 12
    rs = np.random.default_rng(4)
    m = L.simple_cubic_periodic(Lc, onsite=rs.uniform(-8.25, 8.25, Lc ** 3), dtype=dtype)
    h = m.hamiltonian
    sites = np.sort(rs.choice(h.shape[0], 64, replace=False))
    energy = np.linspace(-10, 10, 41)
    rng = (-15.0, 15.0)
    eng = _native.Engine(h, _native.make_config(energy_range=rng))
    got = eng.calc_ldos(sites, energy, 0.25)
    eng.close()
    ref = oracle.core_ldos(h.astype(np.float64), sites, energy, 0.25, energy_range=rng) * PI_RATIO
    err = rel_err(got, ref)
    print("3D Anderson LDOS %s (64 sites): %.3e" % (np.dtype(dtype).name, err))
    assert err <= tol


@pytest.mark.parametrize("precision,tol", [("fp32p", 4e-7), ("fp32", 2e-6)])
def test_fma_compensated_rows_match_the_oracle_on_a_ragged_batch(oracle, precision, tol):
    """precision fp32p: FP32 vectors whose row sums of H~ x are compensated by one FMA per term,
    on a ragged batch of three flakes (row offsets not multiples of 16), 1026 moments, against
    the FP64 oracle; beside it the chained-FMA rows on the same inputs."""
    hs = [_flake(n, s) for n, s in ((9001, 21), (4003, 22), (12007, 23))]
    rng = (-9.5, 9.5)
    M = 1026
    a, b = oracle.scale(*rng)
    starters = [oracle.random_starters(x.shape[0], 64, np.float32) for x in hs]
    flat = np.concatenate([st.ravel() for st in starters])
    batch = kpm_batch([L.Model(x.astype(np.float32), None) for x in hs], energy_range=rng, precision=precision)
    got = batch.engine.moments_diag(M, flat)
    batch.close()
    for s, x in enumerate(hs):
        r = oracle.optimize(x, [0], [0], a, b)
        ref = oracle.moments_diag(r["h2"], oracle.reorder_vector(starters[s].astype(np.float64), r["reorder_map"]), M,
                                  slices=r["slices"])
        err = rel_err(got[s], ref)
        print("%s system %d: %.3e" % (precision, s, err))
        assert err <= tol


@pytest.mark.parametrize("nvec", [64, 16, 1])
def test_compensated_rows_match_the_oracle_on_a_ragged_batch(oracle, nvec):
    """precision fp32x: FP32 vectors whose row sums of H~ x are compensated (error-free products,
    TwoSum) and rounded once, on a ragged batch of three disordered flakes (row offsets not
    multiples of 16), first call and replayed recursion graph, against the FP64 oracle."""
    hs = [_flake(n, s).astype(np.float32) for n, s in ((9001, 21), (4003, 22), (12007, 23))]
    rng = (-9.5, 9.5)
    M = 258
    a, b = oracle.scale(*rng)
    starters = [oracle.random_starters(h.shape[0], nvec, np.float32) for h in hs]
    flat = np.concatenate([st.ravel() for st in starters])
    batch = kpm_batch([L.Model(h, None) for h in hs], energy_range=rng, precision="fp32x")
    got = [batch.engine.moments_diag(M, flat), batch.engine.moments_diag(M, flat)]
    batch.close()
    for s, h in enumerate(hs):
        r = oracle.optimize(h.astype(np.float64), [0], [0], a, b)
        ref = oracle.moments_diag(r["h2"], oracle.reorder_vector(starters[s].astype(np.float64), r["reorder_map"]), M,
                                  slices=r["slices"])
        for k in (0, 1):
            err = rel_err(got[k][s], ref)
            print("fp32x K=%d system %d call %d: %.3e" % (nvec, s, k, err))
            assert err <= 1e-7


@pytest.mark.parametrize("dtype,nvec,tol", [(np.float32, 64, 1e-6), (np.float64, 16, 1e-10),
                                            (np.complex64, 32, 1e-6), (np.complex128, 8, 1e-10),
                                            (np.float32, 1, 1e-6)])
def test_prefetched_entries_step_matches_plain_step_and_oracle(oracle, dtype, nvec, tol):
    """The diagonal step with each warp's ELL entries staged in shared memory a chunk ahead
    (staging="prefetch") against the per-row-load step and the FP64 oracle, on a ragged batch of
    three flakes whose sizes are not multiples of the 16-row chunks; then the same with the
    optimal-size row limits of an LDOS (tiles cut at shrinking row counts)."""
    hs = [_flake(n, s) for n, s in ((9001, 1), (4003, 2), (12007, 3))]
    if np.iscomplexobj(np.zeros(1, dtype)):
        hs = [(h + 1j * sp.triu(h, 1) * 0.1 - 1j * sp.tril(h, -1) * 0.1).tocsr() for h in hs]
    hs = [h.astype(dtype) for h in hs]
    rng = (-9.5, 9.5)
    M = 130
    a, b = oracle.scale(*rng)
    starters = [oracle.random_starters(h.shape[0], nvec, dtype) for h in hs]
    flat = np.concatenate([st.ravel() for st in starters])
    out = {}
    for staging in ("prefetch", "registers"):
        batch = kpm_batch([L.Model(h, None) for h in hs], energy_range=rng, staging=staging)
        out[staging] = batch.engine.moments_diag(M, flat)
        assert (batch.engine.stats().prefetch > 0) == (staging == "prefetch")
        out[staging + "2"] = batch.engine.moments_diag(M, flat)  # replayed recursion graph
        batch.close()
    for s, h in enumerate(hs):
        h64 = h.astype(np.complex128 if np.iscomplexobj(h.data) else np.float64)
        r = oracle.optimize(h64, [0], [0], a, b)
        ref = oracle.moments_diag(r["h2"], oracle.reorder_vector(starters[s].astype(h64.dtype), r["reorder_map"]), M,
                                  slices=r["slices"])
        for k in ("prefetch", "prefetch2", "registers"):
            err = rel_err(out[k][s], ref)
            print("%s K=%d %s system %d: %.3e" % (np.dtype(dtype).name, nvec, k, s, err))
            assert err <= tol
    # LDOS with optimal-size row limits, 8 sites of the first flake
    h = hs[0]
    sites = np.arange(0, h.shape[0], h.shape[0] // 8)[:8]
    energy = np.linspace(-1, 1, 11)
    res = {}
    for staging in ("prefetch", "registers"):
        eng = _native.Engine(h, _native.make_config(energy_range=rng, staging=staging))
        res[staging] = eng.calc_ldos(sites, energy, 0.1)
        eng.close()
    ref = oracle.core_ldos(h.astype(np.complex128 if np.iscomplexobj(h.data) else np.float64), sites, energy, 0.1,
                           energy_range=rng) * PI_RATIO
    for k, v in res.items():
        err = rel_err(v, ref)
        print("  LDOS %s: %.3e" % (k, err))
        assert err <= tol


def _flake(n_sites, seed):
    m = L.graphene_flake(n_sites, onsite_modifiers=[L.anderson_disorder(1.0, seed)])
    return m.hamiltonian.astype(np.float64)


def test_cpp_host_caller_runs_on_the_gpu():
    """tests/cpp/host_caller.cpp: a C++ program calling the engine through the C ABI only
    (create, scaling factors, diagonal moments of unit starters on a ring, stats, destroy)
    reproduces the ring's closed-form moments in FP64, complex128 and FP32."""
    import os
    import subprocess
    from pybinding_gb300 import build
    from tests.conftest import ROOT
    exe = build.build_host_program(os.path.join(ROOT, "tests", "cpp", "host_caller.cpp"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all checks passed" in r.stdout


def test_progress_callback_follows_the_reference_protocol():
    """progress_callback(delta, total) during calc_dos (kpm/default/Compute.cpp:64-87,133-144):
    (-1, total) first, then increments adding up to total, then (total, total); nothing with
    silent=True; the moments are those of a call without reporting."""
    m = L.graphene_flake(20000, onsite_modifiers=[L.anderson_disorder(1.0, 3)])
    calls = []
    energy = np.linspace(-2, 2, 41)
    k = kpm(m, energy_range=(-9.0, 9.0), progress_callback=lambda d, t: calls.append((d, t)))
    dos = k.calc_dos(energy, 0.05, num_random=16).data
    assert calls[0] == (-1, 16) and calls[-1] == (16, 16)
    inc = [d for d, _ in calls[1:-1]]
    assert sum(inc) == 16 and all(d >= 0 for d in inc) and len(inc) > 1, calls
    quiet = kpm(m, energy_range=(-9.0, 9.0), silent=True)
    np.testing.assert_allclose(quiet.calc_dos(energy, 0.05, num_random=16).data, dos, rtol=1e-12, atol=0)
    print("progress calls:", calls)
