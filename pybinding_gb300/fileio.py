"""``pb.save`` / ``pb.load``: results in pybinding's ``.pbz`` files.

The format: a ``.pbz`` file is one pickle (protocol 4) inside a gzip stream. A file
name given without any extension is stored with ``.pbz`` appended, and loading a name
that does not exist falls back to the same name with ``.pbz`` appended
(``pybinding/support/pickle.py:39-74`` defines this behaviour). Result classes
pickle their state as the mapping ``{"version": v, "dict": attributes}``
(``pybinding/support/pickle.py:77-106``).

Files written by pybinding load here as well: numpy arrays and plain Python data as
they are, and pybinding's ``results.Series``, ``Sweep`` and ``NDSweep`` as this
package's classes of the same names and attributes. Other pybinding classes have no
counterpart in this package and raise ``pickle.UnpicklingError`` naming the class.
"""
from __future__ import annotations

import gzip
import os
import pickle

__all__ = ["save", "load"]

SUFFIX = ".pbz"
PICKLE_PROTOCOL = 4


class Versioned:
    """Pickled state ``{"version": 0, "dict": attributes}``, the layout of pybinding's result
    classes, so that a result saved by either package carries the same state."""

    STATE_VERSION = 0

    def __getstate__(self):
        return {"version": self.STATE_VERSION, "dict": self.__dict__}

    def __setstate__(self, state):
        if "version" not in state:  # a plain attribute dictionary
            self.__dict__.update(state)
            return
        if state["version"] != self.STATE_VERSION:
            raise RuntimeError("%s pickles state version %d; this file holds version %s" % (
                type(self).__name__, self.STATE_VERSION, state["version"]))
        self.__dict__.update(state["dict"])


def _is_stream(file):
    return hasattr(file, "read") or hasattr(file, "write")


def _target(file):
    """The path to write: ``file`` itself, or ``file + '.pbz'`` when it has no extension."""
    name = os.fspath(file)
    return name if os.path.splitext(name)[1] else name + SUFFIX


def _source(file):
    """The path to read: ``file`` if it exists, else the ``.pbz`` name that saving it would use."""
    name = os.fspath(file)
    if os.path.exists(name):
        return name
    alt = _target(name)
    return alt if os.path.exists(alt) else name


def save(obj, file):
    """Write ``obj`` as a gzip-compressed pickle (a path or a binary file object)."""
    if _is_stream(file):
        with gzip.GzipFile(fileobj=file, mode="wb") as z:
            pickle.dump(obj, z, protocol=PICKLE_PROTOCOL)
        return
    with gzip.GzipFile(_target(file), mode="wb") as z:
        pickle.dump(obj, z, protocol=PICKLE_PROTOCOL)


# pybinding's result classes, by their pickled (module, name), and this package's equivalents
_PYBINDING_RESULTS = {"Series": ("chebyshev", "Series"), "Sweep": ("parallel", "Sweep"),
                      "NDSweep": ("parallel", "NDSweep")}


class _ResultUnpickler(pickle.Unpickler):
    def find_class(self, module, name):
        top = module.partition(".")[0]
        if top not in ("pybinding", "_pybinding"):
            return super().find_class(module, name)
        if module == "pybinding.results" and name in _PYBINDING_RESULTS:
            import importlib
            sub, cls = _PYBINDING_RESULTS[name]
            return getattr(importlib.import_module("." + sub, __package__), cls)
        raise pickle.UnpicklingError("%s.%s has no counterpart in pybinding_gb300" % (module, name))


def load(file):
    """Read an object written by :func:`save` or by pybinding's ``pb.save``."""
    if _is_stream(file):
        with gzip.GzipFile(fileobj=file, mode="rb") as z:
            return _ResultUnpickler(z).load()
    with gzip.GzipFile(_source(file), mode="rb") as z:
        return _ResultUnpickler(z).load()
