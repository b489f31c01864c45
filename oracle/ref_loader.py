"""Import the unmodified OpenBTE reference solver in a container without its GUI/IO deps.

Test and measurement infrastructure only: it generates the golden fixtures
under ``tests/golden``, backs CPU tests that are skipped when the reference is
absent, and runs the reference's own solver for ``bench.py --impl reference``.
It never runs on the product path.

Where the reference lives: ``OBTE_REFERENCE`` (a directory holding
``openbte/bte.py``), else ``baseline/_ref`` in this checkout, which is where
``pip install --no-deps --target baseline/_ref <reference checkout>`` puts the
unmodified package.

The reference (romanodev/OpenBTE 3.0.16) imports shapely, sqlitedict,
pickle5, plotly, jax, icosphere, nptyping, matplotlib and cachetools at module
level, none of which the transport path uses. This loader:

1. registers stub modules for them (a working ``cachetools`` LRU/``cached``);
2. sets ``scipy.interpolate.interp2d`` (removed in scipy>=1.14; imported at
   openbte/objects.py:10);
3. registers a bare ``openbte`` package pointing at the reference sources, which
   skips ``pkg_resources.require`` in openbte/__init__.py:24;
4. pads 2-vectors in ``np.cross`` (numpy>=2 rejects them; openbte/mesh.py:186);
5. re-executes ``Mesh.gradient`` without its dead dense ``(n, n, k)`` allocation
   (openbte/objects.py:328), which is otherwise 80 GiB at 60k cells;
6. sets ``sys.dont_write_bytecode`` so nothing is written into the reference tree;
7. replaces ``utils.run`` (openbte/utils.py:186-219) by an in-process runner with
   the same ``SharedMemory`` semantics (one worker), or leaves the forking
   runner in place with ``n_process`` workers.
"""
from __future__ import annotations

import importlib
import inspect
import os
import sys
import textwrap
import types

import numpy as np

_CHECKOUT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_ROOT = os.environ.get("OBTE_REFERENCE") or os.path.join(_CHECKOUT, "baseline", "_ref")


def available() -> bool:
    return os.path.isfile(os.path.join(REF_ROOT, "openbte", "bte.py"))


def available_inverse() -> bool:
    """The inverse-design modules are present (a pip install of the reference leaves them out: the
    ``openbte/inverse`` folder has no ``__init__.py``, so only a source checkout has them)."""
    return os.path.isfile(os.path.join(REF_ROOT, "openbte", "inverse", "matinverse.py"))


def _stub(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    sys.modules[name] = m
    return m


class _Anything:
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, item):
        return _Anything()

    def __getitem__(self, item):
        return _Anything()


def _install_stubs():
    sys.dont_write_bytecode = True
    for name in ["shapely", "shapely.geometry", "shapely.ops", "shapely.affinity"]:
        _stub(name, Polygon=_Anything, Point=_Anything, MultiPolygon=_Anything,
              unary_union=_Anything(), translate=_Anything())
    _stub("sqlitedict", SqliteDict=_Anything)
    import pickle
    sys.modules["pickle5"] = pickle
    _stub("plotly")
    _stub("plotly.graph_objs")
    jax = _stub("jax", numpy=_Anything(), jit=lambda f=None, **k: f, custom_vjp=_Anything,
                value_and_grad=_Anything())
    _stub("jax.numpy")
    jax.numpy = sys.modules["jax.numpy"]
    _stub("icosphere", icosphere=_Anything())
    _stub("nptyping", NDArray=_Anything(), Shape=_Anything(), Float=float, Int=int)
    _stub("matplotlib")
    _stub("matplotlib.pylab")

    class LRUCache(dict):
        def __init__(self, maxsize=128, **k):
            super().__init__()
            self.maxsize = int(maxsize)

    def cached(cache):
        def deco(f):
            def wrapper(*args):
                if args in cache:
                    return cache[args]
                v = f(*args)
                if len(cache) >= cache.maxsize:
                    cache.pop(next(iter(cache)))
                cache[args] = v
                return v
            return wrapper
        return deco

    _stub("cachetools", LRUCache=LRUCache, cached=cached)
    import scipy.interpolate
    if not hasattr(scipy.interpolate, "interp2d"):
        scipy.interpolate.interp2d = None

    _cross = np.cross
    if not getattr(np.cross, "_obte_padded", False):
        def cross(a, b, *args, **kw):
            a = np.asarray(a)
            b = np.asarray(b)
            if a.shape[-1] == 2:
                a = np.concatenate([a, np.zeros(a.shape[:-1] + (1,))], axis=-1)
            if b.shape[-1] == 2:
                b = np.concatenate([b, np.zeros(b.shape[:-1] + (1,))], axis=-1)
            return _cross(a, b, *args, **kw)
        cross._obte_padded = True
        np.cross = cross


_LOADED = {}


def load(in_process: bool = True):
    """Return the reference modules as a namespace: mesh, bte, fourier, objects, material, utils."""
    if "ns" in _LOADED:
        return _LOADED["ns"]
    if not available():
        raise RuntimeError(f"reference checkout not found at {REF_ROOT}")
    _install_stubs()
    pkg = types.ModuleType("openbte")
    pkg.__path__ = [os.path.join(REF_ROOT, "openbte")]
    sys.modules["openbte"] = pkg
    pkg.Geometry = _Anything
    utils = importlib.import_module("openbte.utils")
    objects = importlib.import_module("openbte.objects")
    pkg.utils = utils
    pkg.objects = objects

    # Mesh.gradient without the dead dense allocation
    src = textwrap.dedent(inspect.getsource(objects.Mesh.gradient))
    src = "\n".join(l for l in src.splitlines() if "A = np.zeros((self.n_elems,self.n_elems" not in l)
    g = {"np": np, "BoundaryConditions": objects.BoundaryConditions}
    exec(compile(src, "<Mesh.gradient>", "exec"), g)
    objects.Mesh.gradient = g["gradient"]

    mesh = importlib.import_module("openbte.mesh")
    material = importlib.import_module("openbte.material")
    bte = importlib.import_module("openbte.bte")
    fourier = importlib.import_module("openbte.fourier")

    if in_process:
        def run(target, n_tasks, shared_variables={}):
            sh = objects.SharedMemory(1)
            for name, value in shared_variables.items():
                sh[name] = value
            inds = [np.arange(n) for n in n_tasks]
            target(sh, inds)
            return sh
        utils.run = run

    ns = types.SimpleNamespace(mesh=mesh, bte=bte, fourier=fourier, objects=objects,
                               material=material, utils=utils)
    _LOADED["ns"] = ns
    return ns


# ---- the inverse-design modules (openbte/inverse/bte.py, openbte/inverse/matinverse.py) ----------
#
# They use jax only as an array library (jnp.einsum / zeros / power, functional ``.at[].add``) and
# for ``jit`` / ``custom_vjp`` decorators; the gradient itself is written out by hand
# (openbte/inverse/bte.py:27-95).  jax is absent here, so ``jax.numpy`` is replaced by a numpy
# module whose arrays support ``.at[idx].add(v)`` (np.add.at on a copy) and the decorators become
# identities.  The arithmetic is then the reference's own, in float64 (it enables jax x64,
# openbte/inverse/matinverse.py:33).

class _JArr(np.ndarray):
    @property
    def at(self):
        return _At(self)


class _At:
    def __init__(self, a):
        self.a = a

    def __getitem__(self, idx):
        return _AtIdx(self.a, idx)


class _AtIdx:
    def __init__(self, a, idx):
        self.a, self.idx = a, idx

    def add(self, v):
        out = np.array(self.a, dtype=np.result_type(self.a, np.asarray(v)), copy=True)
        np.add.at(out, self.idx, np.asarray(v))
        return out.view(_JArr)

    def set(self, v):
        out = np.array(self.a, copy=True)
        out[self.idx] = np.asarray(v)
        return out.view(_JArr)


def _w(x):
    return np.asarray(x).view(_JArr)


def _numpy_jax():
    jnp = types.ModuleType("jax.numpy")
    for name in ["array", "zeros", "ones", "einsum", "power", "multiply", "sqrt", "concatenate", "fliplr",
                 "zeros_like", "ones_like", "arange", "exp", "sum", "linalg"]:
        f = getattr(np, name)
        if callable(f):
            jnp.__dict__[name] = (lambda f: (lambda *a, **k: _w(f(*a, **k))))(f)
        else:
            jnp.__dict__[name] = f
    jnp.allclose = np.allclose
    jnp.dot = lambda *a, **k: _w(np.dot(*a, **k))
    jnp.float64 = np.float64
    jax = types.ModuleType("jax")
    jax.numpy = jnp
    jax.jit = lambda f=None, **k: f if f is not None else (lambda g: g)
    jax.custom_vjp = lambda f: f
    jax.value_and_grad = lambda f, **k: f
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
    jsig = types.ModuleType("jax.scipy.signal")
    jsig.convolve2d = None
    jsc = types.ModuleType("jax.scipy")
    jsc.signal = jsig
    jax.scipy = jsc
    return {"jax": jax, "jax.numpy": jnp, "jax.scipy": jsc, "jax.scipy.signal": jsig}


def load_inverse():
    """Return the reference's inverse-design modules (bte, matinverse) on the numpy jax stand-in."""
    if "inv" in _LOADED:
        return _LOADED["inv"]
    load()
    saved = {k: sys.modules.get(k) for k in ["jax", "jax.numpy", "jax.scipy", "jax.scipy.signal"]}
    sys.modules.update(_numpy_jax())
    mpl = sys.modules["matplotlib"]
    mpl.interactive = lambda *a, **k: None
    mpl.rcParams = {}
    sys.modules["matplotlib.pylab"].__dict__.setdefault("figure", _Anything())
    _stub("nlopt")
    pkg = sys.modules["openbte"]
    inv = types.ModuleType("openbte.inverse")
    inv.__path__ = [os.path.join(REF_ROOT, "openbte", "inverse")]
    sys.modules["openbte.inverse"] = inv
    pkg.inverse = inv
    try:
        mi = importlib.import_module("openbte.inverse.matinverse")
        ib = importlib.import_module("openbte.inverse.bte")
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    ns = types.SimpleNamespace(bte=ib, matinverse=mi, asarray=_w)
    _LOADED["inv"] = ns
    return ns
