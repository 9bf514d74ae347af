"""The C ABI library builds, loads and exports every entry point of include/*.h.

These run without a GPU: only host-side entry points are called (argument
checks, kernel damping coefficients), never the recursion.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest
import scipy.sparse as sp

from pybinding_gb300 import _native

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
HEADERS = sorted(os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h"))


def declared_functions():
    names = set()
    for header in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(header).read(), flags=re.S)
        names |= set(re.findall(r"^[A-Za-z_][\w\s\*]*?\b(kpm_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_header_declares_the_abi():
    names = declared_functions()
    assert "kpm_create" in names and "kpm_moments_diag" in names and "kpm_calc_dos" in names
    assert "kpm_lattice_honeycomb" in names and "kpm_lattice_csr" in names
    assert len(names) >= 26


def test_library_exports_every_declared_symbol():
    lib = _native.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared_functions()) <= set(_native.SIGNATURES), "binding table lacks a declared function"


def test_damping_matches_oracle(oracle):
    for kern, lam in (("jackson", 4.0), ("lorentz", 4.0), ("lorentz", 3.0), ("dirichlet", 4.0)):
        for n in (2, 10, 2050):
            np.testing.assert_array_equal(_native.damping_coefficients(kern, lam, n), oracle.damping(kern, lam, n))
    for sb in (0.0174, 0.05, 0.0031, 1e-4):
        for kern in ("jackson", "lorentz", "dirichlet"):
            assert _native.required_num_moments(kern, 4.0, sb) == oracle.required_num_moments(kern, 4.0, sb)


def test_round_num_moments(oracle):
    for n in range(0, 40):
        assert _native.round_num_moments(n) == oracle.round_num_moments(n)


def _small_h(dtype=np.float32):
    h = sp.diags([np.ones(9), np.ones(9)], [-1, 1], shape=(10, 10), format="csr").astype(dtype)
    h.sort_indices()
    return h


def _create(h, cfg=None, offsets=None):
    cfg = cfg or _native.make_config()
    ip = np.ascontiguousarray(h.indptr, np.int32)
    ix = np.ascontiguousarray(h.indices, np.int32)
    v = np.ascontiguousarray(h.data)
    off = None if offsets is None else np.ascontiguousarray(offsets, np.int64)
    handle = C.c_void_p()
    rc = _native.lib().kpm_create(_native.SCALAR_CODE[v.dtype], h.shape[0], _native.ptr(ip), _native.ptr(ix),
                                  _native.ptr(v), 1 if off is None else off.size - 1, _native.ptr(off),
                                  C.byref(cfg), C.byref(handle))
    msg = _native.lib().kpm_last_error().decode()
    if rc == 0:
        _native.lib().kpm_destroy(handle)
    return rc, msg


def test_create_rejects_bad_energy_range():
    """kpm/Core.cpp:20-22"""
    rc, msg = _create(_small_h(), _native.make_config(energy_range=(1.0, -1.0)))
    assert rc == _native.KPM_ERR_VALUE and msg == "KPM: Invalid energy range specified (min > max)."


def test_create_rejects_nan():
    """hamiltonian/Hamiltonian.hpp:133-140"""
    h = _small_h(np.float64)
    h.data[3] = np.nan
    rc, msg = _create(h)
    assert rc == _native.KPM_ERR_RUNTIME and "NaN or INF" in msg


def test_create_rejects_bad_csr():
    h = _small_h()
    h.indices[0] = 42
    rc, msg = _create(h)
    assert rc == _native.KPM_ERR_VALUE and "out of range" in msg
    h = _small_h()
    rc, msg = _create(h, offsets=[0, 5, 10])  # hoppings 4<->5 cross the block boundary
    assert rc == _native.KPM_ERR_VALUE and "system block" in msg
    rc, msg = _create(h, offsets=[0, 10, 10])
    assert rc == _native.KPM_ERR_VALUE


def test_lorentz_lambda_checked():
    rc, msg = _create(_small_h(), _native.make_config(kernel="lorentz", kernel_param=-1.0))
    assert rc == _native.KPM_ERR_VALUE and "lambda must be positive" in msg


def test_compute_without_gpu_fails_cleanly():
    """Creating an engine is host-only; the first device call reports a CUDA error."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    eng = _native.Engine(_small_h(), _native.make_config())
    with pytest.raises(RuntimeError, match="CUDA"):
        eng.calc_dos(np.linspace(-1, 1, 5), 0.1, 1)
    eng.close()


def test_optimized_hamiltonian_bit_exact(oracle):
    """The engine's reorder (host C++) equals create_reordered bit for bit
    (kpm/OptimizedHamiltonian.cpp:75-152), f32 and c64, b == 0 and b != 0."""
    from tests import models as TM
    cases = [(TM.cpp_fixture_model(), (-6.25, 8.25)), (TM.cpp_fixture_model_plain(), (-12.0, 10.0)),
             (TM.graphene("magnetic_field", 3), (-8.5, 8.5)), (TM.graphene("const_potential", 3), (-8.0, 9.0))]
    for m, rng in cases:
        h = m.hamiltonian
        eng = _native.Engine(h, _native.make_config(energy_range=rng))
        a, b = oracle.scale(*rng)
        assert eng.scaling_factors() == (a, b)
        n = h.shape[0]
        for src, dest in (([0], [0]), ([n // 2], [n // 3, n // 4]), ([n - 1, 1], [2, n - 2])):
            for reorder in (True, False):
                got = eng.optimized_hamiltonian(src, dest, reorder)
                ref = oracle.optimize(h, src, dest, a, b, reorder)
                assert np.array_equal(got["h2"].indptr, ref["h2"].indptr)
                assert np.array_equal(got["h2"].indices, ref["h2"].indices)
                gv, rv = got["h2"].data, ref["h2"].data
                assert gv.dtype == rv.dtype and np.array_equal(gv.view(np.uint8), rv.view(np.uint8))
                assert np.array_equal(got["reorder_map"], ref["reorder_map"])
                assert np.array_equal(got["slices"], ref["slices"])
                assert np.array_equal(got["src"], ref["src"]) and np.array_equal(got["dest"], ref["dest"])
                assert (got["src_offset"], got["dest_offset"]) == (ref["src_offset"], ref["dest_offset"])
        eng.close()


def test_optimized_hamiltonian_disconnected_bit_exact(oracle):
    """A system of two flakes without a shared bond plus a site with no entries: the reorder
    continues from the first unreached row when the target's component is exhausted (the
    reference assumes a connected graph); engine and oracle agree bit for bit, and every row
    appears exactly once."""
    import scipy.sparse as sp
    from pybinding_gb300 import lattice as L
    h1 = L.graphene_flake(300).hamiltonian
    h2 = L.graphene_flake(200).hamiltonian
    h = sp.block_diag([h1, sp.csr_matrix((1, 1), dtype=h1.dtype), h2], format="csr")
    h.sort_indices()
    n = h.shape[0]
    for rng in ((-9.0, 9.0), (-8.0, 9.5)):
        eng = _native.Engine(h, _native.make_config(energy_range=rng))
        a, b = oracle.scale(*rng)
        for src in ([0], [h1.shape[0] + 5], [h1.shape[0]]):
            got = eng.optimized_hamiltonian(src, src)
            ref = oracle.optimize(h, src, src, a, b)
            assert np.array_equal(np.sort(got["reorder_map"]), np.arange(n))
            assert np.array_equal(got["reorder_map"], ref["reorder_map"])
            assert np.array_equal(got["h2"].indptr, ref["h2"].indptr)
            assert np.array_equal(got["h2"].indices, ref["h2"].indices)
            assert np.array_equal(got["h2"].data.view(np.uint8), ref["h2"].data.view(np.uint8))
            assert np.array_equal(got["slices"], ref["slices"])
        eng.close()


def test_config_fields_are_checked_on_create():
    """kpm_create rejects launch options outside their ranges before touching the GPU."""
    h = _small_h()
    for field, bad, msg in (("staging", 3, "staging must be"), ("fuse_steps", 3, "fuse_steps must be"),
                            ("precision", 7, "unknown precision mode")):
        cfg = _native.make_config()
        setattr(cfg, field, bad)
        with pytest.raises(ValueError, match=msg):
            _native.Engine(h, cfg)
    for staging in ("auto", "registers", "prefetch"):
        _native.Engine(h, _native.make_config(staging=staging)).close()
    with pytest.raises(ValueError, match="Invalid energy range"):
        _native.Engine(h, _native.make_config(energy_range=(1.0, -1.0)))


def test_spatial_ldos_refuses_multi_orbital_models():
    """KPM.cpp:69-71: calc_spatial_ldos raises for multi-orbital models (here a duck-typed model
    with two Hamiltonian rows per site), before any device work."""
    import types
    from pybinding_gb300 import kpm
    h = _small_h()
    n = h.shape[0]
    system = types.SimpleNamespace(x=np.zeros(n // 2, np.float32), y=np.zeros(n // 2, np.float32),
                                   z=np.zeros(n // 2, np.float32), num_sites=n // 2, hamiltonian_size=n)
    system.positions = (system.x, system.y, system.z)
    model = types.SimpleNamespace(hamiltonian=h, system=system)
    k = kpm(model, energy_range=(-1, 1))
    with pytest.raises(RuntimeError, match="doesn't currently support multi-orbital models"):
        k.calc_spatial_ldos(np.linspace(-0.5, 0.5, 3), 0.1, lambda x, y, z: np.ones(x.size, bool))


def test_cpp_host_caller_builds_against_the_c_abi():
    """tests/cpp/host_caller.cpp (a C++ program that calls kpm_create / kpm_moments_diag /
    kpm_destroy through include/kpm_gb300.h) compiles and links against the library; its
    GPU-free first check (the reference's error for min > max) passes before any device use."""
    import subprocess
    from pybinding_gb300 import build
    from tests.conftest import ROOT
    exe = build.build_host_program(os.path.join(ROOT, "tests", "cpp", "host_caller.cpp"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.stdout.startswith("ok: kpm_create rejects min > max"), r.stdout


def test_pybind_module_raises_the_reference_exception_types():
    """The pybind11 module (csrc/pykpm.cpp) over the C ABI: std::invalid_argument-like errors
    come out as ValueError, others as RuntimeError (cppmodule/src/kpm.cpp semantics), unknown
    configuration keys as TypeError; the host-side calls need no GPU."""
    from pybinding_gb300 import _binding
    h = _small_h()
    with pytest.raises(ValueError, match="Invalid energy range"):
        _binding.Engine(h, dict(energy_range=(1.0, -1.0)))
    with pytest.raises(TypeError, match="unknown KPM configuration key"):
        _binding.Engine(h, dict(colour="red"))
    bad = h.copy()
    bad.data[0] = np.nan
    with pytest.raises(RuntimeError, match="invalid values: NaN or INF"):
        _binding.Engine(bad)
    e = _binding.Engine(h, dict(energy_range=(-2.0, 2.0), num_threads=2))
    assert e.rows == 10 and e.num_systems == 1 and e.dtype == np.float32
    a, b = e.scaling_factors()
    assert a == pytest.approx(2.02, rel=1e-6) and b == 0
    np.testing.assert_array_equal(_binding.damping_coefficients("jackson", 4.0, 7),
                                  _native.damping_coefficients("jackson", 4.0, 7))
    assert _binding.round_num_moments(2048) == 2050
    e.close()
    with pytest.raises(RuntimeError, match="closed"):
        e.scaling_factors()


def test_spatial_ldos_refuses_the_three_band_tmd_model():
    """The refusal on a real multi-orbital model (three orbitals per MoS2 site)."""
    from pybinding_gb300 import kpm, lattice as L
    k = kpm(L.build_tmd_3band(L.rectangle(2), "MoS2"), energy_range=(-3, 6), silent=True)
    with pytest.raises(RuntimeError, match="doesn't currently support multi-orbital models"):
        k.calc_spatial_ldos(np.linspace(0, 1, 3), 0.1, lambda x, y, z: np.ones(x.size, bool))

