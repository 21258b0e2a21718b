"""Import the reference bilby package in place, with small stand-ins for the
third-party modules it imports but that this container does not ship.

TEST INFRASTRUCTURE ONLY.  This module is used to generate the golden
fixtures under ``tests/golden/`` and by CPU tests that cross-check the numpy
restatement in :mod:`oracle.restate` against the reference itself.  It needs
the reference source tree: the directory named by ``GWL_REFERENCE_ROOT``, or
else a checkout named ``reference`` beside this repository (``../reference``
from the repository root).  It is never imported by the library, by
``bench.py`` or by any GPU test.

Stand-ins provided (only what the likelihood hot path touches):

* ``array_api_compat``: a numpy-only namespace resolver.
* ``array_api_extra``: ``at(x, idx).set(v)`` returning an updated copy.
* ``plum``: a small multiple-dispatch decorator that selects an overload by
  argument binding and ``isinstance`` checks on annotated parameters, honouring
  ``precedence`` and ``.dispatch`` registration (``bilby/gw/detector/networks.py:487``).
* ``MagicMock`` modules for plotting / IO / sampler packages that are imported
  at module import time but never called on the likelihood path.

``bilby_cython`` is deliberately *not* stubbed: ``bilby/gw/compat/__init__.py``
skips the Cython overrides when the import fails, which leaves the
pure-Python geometry/time code in charge (the code the oracle restates).
"""
from __future__ import annotations

import inspect
import os
import sys
import types
import typing
from unittest.mock import MagicMock

import numpy as np

_REPO_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE_ROOT = os.environ.get("GWL_REFERENCE_ROOT") or os.path.normpath(os.path.join(_REPO_ROOT, "..", "reference"))

_INSTALLED = False


def reference_available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "bilby"))


# --------------------------------------------------------------------------
# array_api_compat stand-in (numpy only)
# --------------------------------------------------------------------------
def _make_array_api_compat():
    m = types.ModuleType("array_api_compat")

    def array_namespace(*xs, **kw):
        return np

    m.array_namespace = array_namespace
    m.get_namespace = array_namespace
    m.is_array_api_obj = lambda x: isinstance(x, (np.ndarray, np.generic))
    m.is_numpy_array = lambda x: isinstance(x, (np.ndarray, np.generic))
    m.is_numpy_namespace = lambda xp: xp is np
    for name in ("jax", "torch", "cupy", "dask", "ndonnx", "sparse", "pydata_sparse"):
        setattr(m, f"is_{name}_array", lambda x: False)
        setattr(m, f"is_{name}_namespace", lambda xp: False)
    m.is_array_api_strict_namespace = lambda xp: False
    m.device = lambda x: "cpu"
    m.to_device = lambda x, d, **kw: x
    m.size = lambda x: int(np.size(x))
    m.numpy = np
    return m


def _make_array_api_extra():
    m = types.ModuleType("array_api_extra")

    class _At:
        def __init__(self, x, idx):
            self.x, self.idx = x, idx

        def set(self, v, **kw):
            y = np.array(self.x, copy=True)
            y[self.idx] = v
            return y

        def add(self, v, **kw):
            y = np.array(self.x, copy=True)
            y[self.idx] += v
            return y

        def multiply(self, v, **kw):
            y = np.array(self.x, copy=True)
            y[self.idx] *= v
            return y

    def at(x, idx=None):
        return _At(x, idx)

    m.at = at
    return m


# --------------------------------------------------------------------------
# plum stand-in: multiple dispatch by binding + isinstance on annotations
# --------------------------------------------------------------------------
def _type_ok(value, ann) -> bool:
    if ann is inspect.Parameter.empty or ann is typing.Any:
        return True
    if isinstance(ann, str):
        return True
    try:
        return isinstance(value, ann)
    except TypeError:
        origin = typing.get_origin(ann)
        if origin is typing.Union:
            return any(_type_ok(value, a) for a in typing.get_args(ann))
        return True


class _Function:
    def __init__(self, name):
        self.name = name
        self.methods = []  # (precedence, specificity, signature, func)
        self.__name__ = name

    def register(self, func, precedence=0):
        sig = inspect.signature(func)
        spec = sum(1 for p in sig.parameters.values() if p.annotation is not inspect.Parameter.empty)
        self.methods.append((precedence, spec, sig, func))
        self.methods.sort(key=lambda t: (-t[0], -t[1]))
        if not hasattr(self, "__doc__") or self.__doc__ is None:
            self.__doc__ = func.__doc__
        return self

    def dispatch(self, func=None, *, precedence=0):
        if func is None:
            return lambda f: (self.register(f, precedence), self)[1]
        self.register(func, precedence)
        return self

    def __call__(self, *args, **kwargs):
        for _, _, sig, func in self.methods:
            try:
                bound = sig.bind(*args, **kwargs)
            except TypeError:
                continue
            ok = True
            for name, val in bound.arguments.items():
                p = sig.parameters[name]
                if p.kind in (p.VAR_POSITIONAL, p.VAR_KEYWORD):
                    continue
                if not _type_ok(val, p.annotation):
                    ok = False
                    break
            if ok:
                return func(*args, **kwargs)
        raise TypeError(f"no overload of {self.name} matches the arguments")


def _make_plum():
    m = types.ModuleType("plum")
    registry: dict = {}

    def dispatch(func=None, *, precedence=0):
        def deco(f):
            key = f.__name__
            fn = registry.get(key)
            if fn is None:
                fn = _Function(key)
                registry[key] = fn
            fn.register(f, precedence)
            return fn

        if func is None:
            return deco
        return deco(func)

    m.dispatch = dispatch
    m.Function = _Function
    return m


_MOCKED = [
    "pandas", "matplotlib", "matplotlib.pyplot", "matplotlib.lines", "matplotlib.ticker",
    "matplotlib.colors", "matplotlib.cm", "matplotlib.gridspec", "matplotlib.patches",
    "h5py", "dill", "dynesty", "dynesty.utils", "emcee", "corner", "astropy",
    "astropy.units", "astropy.cosmology", "astropy.time", "astropy.coordinates",
    "astropy.constants", "gwpy", "gwpy.timeseries", "gwpy.frequencyseries",
    "lal", "lalsimulation", "orng", "interpax", "lalframe",
    "ligo", "ligo.skymap", "scipy.stats._qmc", "gwpopulation",
]


def _mock_module(name):
    import importlib.machinery

    mod = MagicMock(name=name)
    mod.__spec__ = importlib.machinery.ModuleSpec(name, loader=None)
    mod.__path__ = []
    return mod


def install():
    """Register the stand-in modules and put the reference on ``sys.path``."""
    global _INSTALLED
    if _INSTALLED:
        return
    if not reference_available():
        raise RuntimeError(f"reference tree not found at {REFERENCE_ROOT}")
    sys.modules.setdefault("array_api_compat", _make_array_api_compat())
    sys.modules.setdefault("array_api_extra", _make_array_api_extra())
    sys.modules.setdefault("plum", _make_plum())
    orng = types.ModuleType("orng")
    orng.RandomGenerator = type("RandomGenerator", (), {})
    sys.modules.setdefault("orng", orng)
    pandas = _mock_module("pandas")
    pandas.Series = type("Series", (), {})
    pandas.DataFrame = type("DataFrame", (), {})
    sys.modules.setdefault("pandas", pandas)
    for name in _MOCKED:
        if name in sys.modules:
            continue
        try:
            if name.startswith("scipy"):
                continue
            __import__(name)
        except Exception:
            sys.modules[name] = _mock_module(name)
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    _INSTALLED = True


def import_bilby():
    """Return the reference ``bilby`` package, imported in place."""
    install()
    import bilby  # noqa: E402

    import logging
    logging.getLogger("bilby").setLevel(logging.ERROR)
    return bilby


def asd_file_path(name: str) -> str:
    return os.path.join(REFERENCE_ROOT, "bilby", "gw", "detector", "noise_curves", name)
