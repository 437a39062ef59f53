"""Import jclsquant's own Python modules -- TEST INFRASTRUCTURE ONLY.

Loads the reference package from its read-only source tree without running
its ``__init__`` (which star-imports the CUDA bridge), with:

* ``jclsquant.cython_modules.blas_funs`` / ``Extra_funs`` bound to the
  modules that ``oracle/build.py`` compiled from the reference's ``.pyx``
  sources into ``oracle/_ref`` (the shipped binaries are never loaded);
* ``matplotlib`` and ``skopt`` stubbed (imported by the reference only for
  plotting and for the thermal optimiser, neither on the KPM path).

Used by ``tests/golden/make_golden.py`` and by CPU tests that pin the oracle
against the live reference.  Nothing here exists on a machine without the
reference tree; callers must check :func:`available` first.
"""
from __future__ import annotations

import importlib
import importlib.util
import os
import sys
import types

from . import build as _build

REFERENCE_PKG = os.path.join(_build.REFERENCE_ROOT, "jclsquant")
_loaded: dict = {}


def available() -> bool:
    return os.path.isdir(REFERENCE_PKG)


def _stub(name: str, **attrs) -> None:
    if name in sys.modules:
        return
    mod = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(mod, k, v)
    sys.modules[name] = mod


def _load_ext(fullname: str, path: str):
    spec = importlib.util.spec_from_file_location(fullname, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[fullname] = mod
    spec.loader.exec_module(mod)
    return mod


def load():
    """Return a namespace with the reference modules used on the KPM path."""
    if _loaded:
        return _loaded["ns"]
    if not available():
        raise RuntimeError("reference source tree is not present on this machine")
    built = _build.build_reference()
    if not built.get("blas_funs") or not built.get("Extra_funs"):
        raise RuntimeError("reference Cython kernels could not be built: %r" % (built,))

    class _Anything(types.ModuleType):
        def __getattr__(self, item):  # any plotting call is a no-op object
            return _Anything(item)

        def __call__(self, *a, **k):
            return _Anything("call")

    plt = _Anything("matplotlib.pyplot")
    _stub("matplotlib", pyplot=plt, ticker=_Anything("matplotlib.ticker"))
    sys.modules.setdefault("matplotlib.pyplot", plt)
    sys.modules.setdefault("matplotlib.ticker", _Anything("matplotlib.ticker"))
    _stub("skopt", gp_minimize=lambda *a, **k: None)

    pkg = types.ModuleType("jclsquant")
    pkg.__path__ = [REFERENCE_PKG]
    sys.modules["jclsquant"] = pkg
    cm = types.ModuleType("jclsquant.cython_modules")
    cm.__path__ = [os.path.join(REFERENCE_PKG, "cython_modules")]
    sys.modules["jclsquant.cython_modules"] = cm
    blas = _load_ext("jclsquant.cython_modules.blas_funs", built["blas_funs"])
    extra = _load_ext("jclsquant.cython_modules.Extra_funs", built["Extra_funs"])
    cm.blas_funs = blas
    cm.Extra_funs = extra

    ns = types.SimpleNamespace()
    for name in ("constants", "hams", "lattice", "ell_matrix", "kernel_and_moments",
                 "recurrence_functions", "modifiers", "observables"):
        setattr(ns, name, importlib.import_module("jclsquant." + name))
    ns.blas_funs = blas
    ns.Extra_funs = extra
    _loaded["ns"] = ns
    return ns
