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
import os
import struct
import tempfile
from concurrent.futures import ProcessPoolExecutor

import numpy as np

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
        _lib.oracle_mirror_to_product.restype = ctypes.c_int
        _lib.oracle_mirror_to_product.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]
        _lib.oracle_adapter_step.restype = ctypes.c_double
        _lib.oracle_adapter_step.argtypes = [ctypes.c_size_t] + [ctypes.c_void_p] * 10
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

    def locate_transport(self, x, y, z, dx, dy, dz, max_steps, nthreads=1):
        """LocateGlobalPoint from the world, then every track transported to the world's
        edge: (located states, the transport() tuple with traces)."""
        st, _ = self.locate(x, y, z, nthreads=nthreads)
        return st, self.transport(x, y, z, dx, dy, dz, st, max_steps, trace=True, nthreads=nthreads)

    def timed_shape_query(self, shape, q, x, y, z, dx=None, dy=None, dz=None, nthreads=1):
        """Wall time (s) of one shape_query call (the batched loop, as the oracle reports)."""
        import time

        t0 = time.perf_counter()
        self.shape_query(shape, q, x, y, z, dx, dy, dz, nthreads=nthreads)
        return time.perf_counter() - t0

    def adapter_step(self, x, y, z, dx, dy, dz, states, step_limit=None):
        """One step per track with the reference-side navigator adapter
        (include/vecgeom_gb300_navigator.hpp) installed on every volume with daughters, through
        its per-track methods (no GPU); returns (out-states, steps)."""
        from .oracle import NAVSTATE_DTYPE, _p

        n = len(x)
        if step_limit is None:
            step_limit = np.full(n, np.finfo(np.float64).max)
        out = np.zeros(n, NAVSTATE_DTYPE)
        step = np.zeros(n)
        self._lib.oracle_adapter_step(n, _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), _p(step_limit), _p(states),
                                      _p(out), _p(step))
        return out, step

    def mirror_to_product(self):
        """The reference-side bridge (include/vecgeom_gb300_mirror.hpp) on this closed
        geometry: a product geometry built from it on the host (vg_geom_build, no GPU).
        Returns the product's info, NavIndex table, BVH arrays per logical volume and shape
        extents, or raises with the placed volume that could not be mirrored."""
        import vecgeom_gb300 as vg

        p = vg.Geometry()
        failed = ctypes.c_int32(-1)
        rc = self._lib.oracle_mirror_to_product(p._h, ctypes.byref(failed))
        if rc != 0:
            raise RuntimeError("mirror failed (%d) at placed volume %d" % (rc, failed.value))
        p.build()
        out = product_summary(p)
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "mirror.geom")
            p.save(path)
            with open(path, "rb") as f:
                out["builder_log"] = f.read()
        return out


def product_summary(p):
    """Host-side contents of a built product geometry, for comparing two builds."""
    def bvh(lv):
        try:
            return p.bvh(lv)
        except Exception:  # a logical volume without daughters has no BVH
            return None

    info = p.info()
    return {"info": info, "nav_table": p.nav_table(), "bvh": [bvh(lv) for lv in range(info["n_lv"])],
            "extents": [p.shape_extent(s) for s in range(info["n_shapes"])]}


# shape codes of the product's builder log (vecgeom_gb300/csrc/vg_types.h ShapeType) where
# the oracle's extern "C" surface numbers them differently (ref_api.cpp oracle_add_shape)
_LOG_TO_ORACLE_SHAPE = {10: 11, 11: 12, 12: 13, 13: 14}


def replay_builder_log(data, geo):
    """Replay a product geometry's saved builder log (vg_geom_save: magic, version, count,
    then (op, arguments...) records as doubles) on an OracleGeometry and close it."""
    n = struct.unpack_from("<Q", data, 12)[0]
    log = np.frombuffer(data, dtype="<f8", count=n, offset=20)
    i = 0
    while i < n:
        op = int(log[i])
        if op == 1:
            t, np_ = int(log[i + 1]), int(log[i + 2])
            geo._shape(_LOG_TO_ORACLE_SHAPE.get(t, t), log[i + 3:i + 3 + np_])
            i += 3 + np_
        elif op == 2:
            geo.add_logical_volume(int(log[i + 1]))
            i += 2
        elif op == 3:
            lv, mother = int(log[i + 1]), int(log[i + 2])
            tr, rot = log[i + 3:i + 6], log[i + 6:i + 15]
            if mother < 0:
                geo.place(lv, tr, rot)
            else:
                geo.place_daughter(mother, lv, tr, rot)
            i += 15
        elif op == 4:
            geo.set_world(int(log[i + 1]))
            i += 2
        else:
            raise ValueError("corrupt builder log")
    geo.close()
    return geo


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


def build_placed_shapes(geo, shapes, placements):
    """Builder for run(): each (kind, params) of `shapes` made as build_shapes does, then
    placed once with the matching (translation, rotation) of `placements`; not closed.
    Returns (shape id, placed-volume id) per shape."""
    from vecgeom_gb300 import workloads as W

    ids = [W.add_shape(geo, kind, params) for kind, params in shapes]
    return [(s, geo.place(geo.add_logical_volume(s), t, r)) for s, (t, r) in zip(ids, placements)]


def build_with_orb(geo):
    """Builder for run(), reference only: a world box holding a box and an Orb (a shape the
    product does not build), closed."""
    world = geo.add_logical_volume(geo.add_box(100.0, 100.0, 100.0))
    geo.place_daughter(world, geo.add_logical_volume(geo.add_box(10.0, 10.0, 10.0)), (-50.0, 0.0, 0.0))
    geo.place_daughter(world, geo.add_logical_volume(geo._shape(15, [20.0])), (50.0, 0.0, 0.0))
    geo.set_world(geo.place(world))
    geo.close()
