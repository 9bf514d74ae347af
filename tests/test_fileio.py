"""``pb.save`` / ``pb.load`` (.pbz files): round trips, and files written by pybinding."""
import contextlib
import gzip
import os
import pathlib
import pickle
import sys
import types

import numpy as np
import pytest

import pybinding_gb300 as pbg
from tests.conftest import GOLDEN


def test_reads_the_reference_kpm_baselines(baselines):
    """The reference's own baseline files (tests/baseline_data/kpm/*.pbz) load unchanged."""
    folder = os.path.join(GOLDEN, "pbz")
    names = sorted(f[:-4] for f in os.listdir(folder) if f.endswith(".pbz"))
    assert len(names) == 9
    for name in names:
        got = pbg.load(os.path.join(folder, name + ".pbz"))
        ref = baselines[name]
        assert got.dtype == ref.dtype and got.shape == ref.shape
        np.testing.assert_array_equal(got, ref)
        # found without the extension too (support/pickle.py:66-70)
        np.testing.assert_array_equal(pbg.load(os.path.join(folder, name)), ref)


def test_save_load_round_trip(tmp_path):
    s = pbg.Series(np.linspace(-1, 1, 7), np.arange(14.0).reshape(7, 2),
                   labels=dict(variable="E (eV)", data="LDOS", columns="orbitals"))
    pbg.save(s, str(tmp_path / "result"))             # no extension: .pbz is added
    assert (tmp_path / "result.pbz").exists()
    for name in (str(tmp_path / "result"), tmp_path / "result.pbz"):
        got = pbg.load(name)
        assert isinstance(got, pbg.Series)
        np.testing.assert_array_equal(got.variable, s.variable)
        np.testing.assert_array_equal(got.data, s.data)
        assert got.labels == s.labels
    with gzip.open(tmp_path / "result.pbz", "rb") as f:   # protocol 4, versioned state
        assert f.read(2) == b"\x80\x04"
    pbg.save({"dos": s, "n": 3}, pathlib.Path(tmp_path / "other.data"))  # an extension is kept
    assert pbg.load(tmp_path / "other.data")["n"] == 3


@contextlib.contextmanager
def _reference_classes(**classes):
    """Register stand-in classes under ``pybinding.results`` while pickling, so that the
    pickle names the reference's classes as a file written by pybinding would."""
    pkg, res = types.ModuleType("pybinding"), types.ModuleType("pybinding.results")
    pkg.results = res
    for name, cls in classes.items():
        cls.__module__, cls.__qualname__ = "pybinding.results", name
        setattr(res, name, cls)
    saved = {k: sys.modules.get(k) for k in ("pybinding", "pybinding.results")}
    sys.modules["pybinding"], sys.modules["pybinding.results"] = pkg, res
    try:
        yield
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v


class _PickleableSeries:
    """State as ``@pickleable`` stores it (support/pickle.py:77-106)."""

    def __getstate__(self):
        return dict(version=0, dict=self.__dict__)


def test_loads_a_series_written_by_pybinding(tmp_path):
    var, data = np.linspace(0, 1, 5), np.random.default_rng(0).random(5).astype(np.float32)
    labels = dict(variable="E (eV)", data="DOS", columns="")
    with _reference_classes(Series=_PickleableSeries):
        s = _PickleableSeries()
        s.variable, s.data, s.labels = var, data, labels
        with gzip.open(tmp_path / "dos.pbz", "wb") as f:
            pickle.dump(s, f, protocol=4)
    got = pbg.load(tmp_path / "dos.pbz")
    assert isinstance(got, pbg.Series)
    np.testing.assert_array_equal(got.variable, var)
    np.testing.assert_array_equal(got.data, data)
    assert got.labels == labels


def test_other_pybinding_classes_are_named_in_the_error(tmp_path):
    class SpatialMap:
        pass

    with _reference_classes(SpatialMap=SpatialMap):
        with gzip.open(tmp_path / "map.pbz", "wb") as f:
            pickle.dump(SpatialMap(), f, protocol=4)
    with pytest.raises(pickle.UnpicklingError, match="pybinding.results.SpatialMap"):
        pbg.load(tmp_path / "map.pbz")


def test_reads_the_reference_sweep_baselines():
    """pybinding's pickled Sweep and NDSweep (tests/baseline_data/parallel/*.pbz) load as
    this package's classes with the reference's attributes, and round-trip."""
    folder = os.path.join(GOLDEN, "pbz_sweeps")
    s = pbg.load(os.path.join(folder, "sweep.pbz"))
    assert isinstance(s, pbg.Sweep)
    assert s.x.shape == (10,) and s.y.shape == (10,) and s.data.shape == (10, 10)
    assert s.labels["title"] == "test sweep" and s.labels["x"] == "V (eV)" and s.labels["data"] == "LDOS"
    nd = pbg.load(os.path.join(folder, "ndsweep.pbz"))
    assert isinstance(nd, pbg.NDSweep)
    assert [len(v) for v in nd.variables] == [5, 4, 10] and nd.data.shape == (5, 4, 10)
    np.testing.assert_array_equal(nd.variables[0], np.linspace(0, 0.1, 5))


def test_sweep_results_round_trip(tmp_path):
    s = pbg.Sweep(np.arange(3.0), np.arange(4.0), np.arange(12.0).reshape(3, 4), labels=dict(x="V"), tags={"a": 1})
    pbg.save(s, tmp_path / "s")
    got = pbg.load(tmp_path / "s")
    assert isinstance(got, pbg.Sweep) and got.labels["x"] == "V" and got.tags == {"a": 1}
    np.testing.assert_array_equal(got.data, s.data)
