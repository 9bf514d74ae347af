"""Generate the committed golden fixtures for the KPM parity tests.

Run from the repository root on a machine that has the pybinding source tree:

    python tests/golden/make_golden.py /path/to/pybinding

It writes these files next to this script:

* ``kpm_baseline.npz`` -- the reference's own golden arrays for its KPM tests
  (``tests/baseline_data/kpm/*.pbz``: gzip-pickled float32 numpy arrays),
  copied verbatim under their test names.
* ``system_baselines.npz`` -- site positions, sublattice site counts and hopping
  pairs of the reference's graphene system baselines (``tests/baseline_data/shape``
  and ``system``: pickled ``System`` objects, read as data without pybinding).
* ``pbz/*.pbz`` -- the KPM baseline files themselves, for the ``.pbz`` reader;
  ``pbz_sweeps/*.pbz`` -- the reference's sweep baselines (pickled ``Sweep`` and
  ``NDSweep`` of deferred KPM LDOS), for the sweep tests.
* ``python_impl_moments.npz`` -- diagonal KPM moments computed by the
  reference's pure-NumPy FP64 implementation (``_PythonImpl`` in
  ``pybinding/chebyshev.py:448-583``) on small Hamiltonians and supplied
  random starters. ``chebyshev.py`` is loaded on its own with stub modules for
  the compiled extension, so the moments come from the reference's code.

The Hamiltonians come from ``pybinding_gb300.lattice`` (a restatement of the
reference builder) and the random starters from the oracle's libstdc++
mt19937 restatement of ``Starter.cpp:48-84``; both are stored in the fixture,
so the tests never rebuild them.
"""
import contextlib
import glob
import gzip
import importlib.util
import os
import pickle
import sys
import types

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def load_reference_chebyshev(ref_root):
    """Import ``pybinding/chebyshev.py`` alone, stubbing its package imports."""
    pkg = types.ModuleType("pybinding")
    pkg.__path__ = []
    stubs = {}
    for name in ["_cpp", "results", "model", "system", "utils", "utils.time", "support", "support.deprecated"]:
        stubs[name] = types.ModuleType("pybinding." + name)
    stubs["model"].Model = type("Model", (), {})
    stubs["system"].System = type("System", (), {})

    class _Timer:
        elapsed = 0.0

    @contextlib.contextmanager
    def timed():
        yield _Timer()

    stubs["utils.time"].timed = timed
    stubs["support.deprecated"].LoudDeprecationWarning = DeprecationWarning
    sys.modules["pybinding"] = pkg
    for name, mod in stubs.items():
        sys.modules["pybinding." + name] = mod
    spec = importlib.util.spec_from_file_location("pybinding.chebyshev",
                                                  os.path.join(ref_root, "pybinding", "chebyshev.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def copy_baselines(ref_root):
    out = {}
    for f in sorted(glob.glob(os.path.join(ref_root, "tests", "baseline_data", "kpm", "*.pbz"))):
        with gzip.open(f, "rb") as fh:
            out[os.path.basename(f)[:-4]] = np.asarray(pickle.load(fh))
    np.savez_compressed(os.path.join(HERE, "kpm_baseline.npz"), **out)
    return out


class _Data:
    """Stand-in for any pybinding class while unpickling a baseline: keeps its state only."""

    def __setstate__(self, state):
        self.state = state


class _DataUnpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if module.split(".")[0] in ("pybinding", "_pybinding"):
            return type(name, (_Data,), {})
        return super().find_class(module, name)


# the reference's system baselines of nearest-neighbour graphene (monolayer lattice) cut
# by a polygon: the shapes of tests/test_shape.py:8-14 and hexagon_ac of tests/test_system.py:8
SYSTEM_CASES = ["shape/polygon_expected[triangle]", "shape/polygon_expected[triangle90]",
                "shape/polygon_expected[diamond]", "shape/polygon_expected[square]",
                "shape/polygon_expected[pentagon]", "system/expected[graphene-monolayer]"]


def copy_system_baselines(ref_root):
    """Site positions, per-sublattice site counts and nearest-neighbour hopping pairs of the
    reference's graphene system baselines (``System`` objects pickled by its tests)."""
    out = {}
    for case in SYSTEM_CASES:
        with gzip.open(os.path.join(ref_root, "tests", "baseline_data", case + ".pbz"), "rb") as fh:
            system = _DataUnpickler(fh).load()
        impl = system.state if isinstance(system.state, dict) else system.state.state
        x, y, z = impl["positions"].state
        rows, cols = impl["hopping_blocks"].state["data"][0]
        key = case.split("/")[1]
        out[key + "/x"], out[key + "/y"], out[key + "/z"] = x, y, z
        out[key + "/site_counts"] = np.asarray(impl["compressed_sublattices"].state["site_counts"])
        out[key + "/hop_rows"], out[key + "/hop_cols"] = np.asarray(rows), np.asarray(cols)
    np.savez_compressed(os.path.join(HERE, "system_baselines.npz"), **out)
    return out


def copy_kpm_pbz(ref_root):
    """The KPM baseline files themselves (a few hundred bytes each), for the .pbz reader, and
    the two sweep baselines (pickled ``Sweep`` / ``NDSweep`` of deferred KPM LDOS,
    tests/test_parallel.py:14-50)."""
    dst = os.path.join(HERE, "pbz")
    os.makedirs(dst, exist_ok=True)
    for f in sorted(glob.glob(os.path.join(ref_root, "tests", "baseline_data", "kpm", "*.pbz"))):
        with open(f, "rb") as src, open(os.path.join(dst, os.path.basename(f)), "wb") as out:
            out.write(src.read())
    dst = os.path.join(HERE, "pbz_sweeps")
    os.makedirs(dst, exist_ok=True)
    for name in ("sweep.pbz", "ndsweep.pbz"):
        with open(os.path.join(ref_root, "tests", "baseline_data", "parallel", name), "rb") as src, \
                open(os.path.join(dst, name), "wb") as out:
            out.write(src.read())


def python_impl_cases(cheb):
    from pybinding_gb300 import lattice as L
    from oracle import oracle as O

    impl = cheb._PythonImpl(model=None, energy_range=(0, 0), kernel=None)
    cases = {}

    def add(tag, model, num_vectors, num_moments):
        h = model.hamiltonian.tocsr()
        h.sort_indices()
        emin, emax, _ = O.lanczos(h.astype(np.complex128 if np.iscomplexobj(h.data) else np.float64))
        # bounds as float32 values: kpm::Config stores energy_range as float, so a
        # user-given range reproduces exactly these scale factors
        emin, emax = float(np.float32(emin - 0.01)), float(np.float32(emax + 0.01))
        a, b = O.scale(emin, emax)
        # the reference's own rescale, in FP64 (chebyshev.py:493-496)
        dt = np.complex128 if np.iscomplexobj(h.data) else np.float64
        h64 = h.astype(dt)
        h2 = sp.csr_matrix(impl._rescale_hamiltonian(h64, a, b))
        h2.sort_indices()
        starters = O.random_starters(h.shape[0], num_vectors, dt)
        mom = np.array([impl._compute_diagonal_moments(num_moments, s, h2) for s in starters])
        cases[tag + "_indptr"] = h64.indptr.astype(np.int32)
        cases[tag + "_indices"] = h64.indices.astype(np.int32)
        cases[tag + "_data"] = h64.data
        cases[tag + "_ab"] = np.array([a, b])
        cases[tag + "_bounds"] = np.array([emin, emax])
        cases[tag + "_starters"] = starters
        cases[tag + "_moments"] = mom

    # complex128: Peierls phases, random-phase starters (the plain-FP64 DOS form)
    add("c128", L.build_honeycomb(L.rectangle(4.0), hopping_modifiers=[L.constant_magnetic_field(200)],
                                  is_complex=True, is_double=True), 4, 130)
    # float64: onsite disorder so that b != 0, Rademacher starters
    add("f64", L.build_honeycomb(L.rectangle(4.0, 3.0), onsite_modifiers=[L.anderson_disorder(1.0, 7)],
                                 is_double=True), 3, 98)
    np.savez_compressed(os.path.join(HERE, "python_impl_moments.npz"), **cases)
    return cases


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PYBINDING_SRC", "")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py /path/to/pybinding [systems]")
    if sys.argv[2:] == ["systems"]:  # only the system baselines and the .pbz copies
        print("system baselines:", sorted({k.split("/")[0] for k in copy_system_baselines(ref)}))
        copy_kpm_pbz(ref)
        sys.exit(0)
    copy_system_baselines(ref)
    copy_kpm_pbz(ref)
    base = copy_baselines(ref)
    print("baselines:", {k: v.shape for k, v in base.items()})
    cheb = load_reference_chebyshev(ref)
    cases = python_impl_cases(cheb)
    print("python impl cases:", sorted(k for k in cases if k.endswith("_moments")))
