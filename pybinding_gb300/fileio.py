"""``pb.save`` / ``pb.load``: results in pybinding's ``.pbz`` files.

A ``.pbz`` file is a gzip-compressed pickle (protocol 4); names without an extension
get ``.pbz`` appended on save and are found with it on load
(``pybinding/support/pickle.py:39-74``). Result classes pickle their state as
``{"version": v, "dict": __dict__}`` (``pybinding/support/pickle.py:77-106``).

Files written by pybinding load here as well: numpy arrays and plain Python data as
they are, and pybinding's ``results.Series``, ``Sweep`` and ``NDSweep`` as this
package's classes of the same names and attributes. Other pybinding classes have no
counterpart in this package and raise ``pickle.UnpicklingError`` naming the class.
"""
from __future__ import annotations

import gzip
import os
import pathlib
import pickle

__all__ = ["save", "load"]


def _normalize(file):
    if isinstance(file, pathlib.PurePath):
        return str(file)
    return file


def _add_extension(file):
    if not isinstance(file, str):
        return file
    path = pathlib.Path(file)
    return str(path.with_suffix(".pbz")) if not path.suffix else file


def save(obj, file):
    """Save ``obj`` to a gzip-compressed pickle; ``.pbz`` is added to a name without extension."""
    file = _add_extension(_normalize(file))
    with gzip.open(file, "wb") as f:
        pickle.dump(obj, f, protocol=4)


def _pybinding_classes():
    from .chebyshev import Series
    from .parallel import NDSweep, Sweep
    return {("pybinding.results", "Series"): Series, ("pybinding.results", "Sweep"): Sweep,
            ("pybinding.results", "NDSweep"): NDSweep}


class _Unpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if module.split(".")[0] in ("pybinding", "_pybinding"):
            cls = _pybinding_classes().get((module, name))
            if cls is None:
                raise pickle.UnpicklingError("%s.%s has no counterpart in pybinding_gb300" % (module, name))
            return cls
        return super().find_class(module, name)


def load(file):
    """Load an object saved by :func:`save` or by pybinding's ``pb.save``."""
    file = _normalize(file)
    file_ext = _add_extension(file)
    if isinstance(file, str) and not os.path.exists(file) and os.path.exists(file_ext):
        file = file_ext
    with gzip.open(file, "rb") as f:
        return _Unpickler(f).load()
