"""The compiled reference (TEST INFRASTRUCTURE ONLY): the reference's own C++ sources built by
oracle/build_ref.py into oracle/_ref/libvgref.so, driven through OracleGeometry's interface,
so that the same builder function (vecgeom_gb300.workloads) and the same queries run on the
reference's code and on the hand-written oracle, and the two are compared.

The reference keeps one geometry per process (GeoManager and the navigation index table are
singletons), so every use goes through `run()`, which builds the geometry and runs the
requested calls in a fresh process and returns their results.
"""
import ctypes
import importlib
import multiprocessing as mp
from concurrent.futures import ProcessPoolExecutor

from . import build_ref
from .oracle import OracleGeometry, bind

_lib = None


def available():
    """True where the reference tree is present to build from (not on a machine that has
    only this repository)."""
    return build_ref.available()


def load():
    global _lib
    if _lib is None:
        _lib = bind(ctypes.CDLL(build_ref.build()), required=False)
    return _lib


class ReferenceGeometry(OracleGeometry):
    """OracleGeometry's construction and query surface on the reference's own code
    (placed and unplaced shape queries, LocateGlobalPoint, ComputeStepAndPropagatedState,
    ComputeStepAndSafetyAndPropagatedState, the navigation index table)."""

    def __init__(self):
        self._lib = load()
        self._h = self._lib.oracle_geom_create()
        if not self._h:
            raise RuntimeError("the reference holds one geometry per process")

    def __del__(self):
        self._h = None


def _worker(builder, builder_kwargs, calls):
    mod, name = builder
    g = ReferenceGeometry()
    getattr(importlib.import_module(mod), name)(g, **builder_kwargs)
    out = []
    for method, args, kwargs in calls:
        out.append(getattr(g, method)(*args, **kwargs))
    return out


def run(builder, calls, builder_kwargs=None):
    """Build a geometry with `builder` = (module, function name), called as
    function(geometry, **builder_kwargs) (it must close the geometry), then run each
    (method, args, kwargs) of `calls` on it, in a fresh process; returns the results."""
    build_ref.build()  # once, in this process, so that workers never race to build
    with ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as pool:
        return pool.submit(_worker, builder, builder_kwargs or {}, calls).result()


def build_gdml(geo, path):
    """Builder for run(): the GDML file at `path` (vecgeom_gb300.gdml), closed."""
    from vecgeom_gb300 import gdml

    gdml.load(path, geo)


def build_shapes(geo, shapes):
    """Builder for run(): each (kind, params) of `shapes` made with
    vecgeom_gb300.workloads.add_shape (boolean operands placed first); not closed."""
    from vecgeom_gb300 import workloads as W

    for kind, params in shapes:
        W.add_shape(geo, kind, params)
