"""Loader of tests/golden/reference_outputs.npz (outputs of the reference's own code, with
the inputs they were computed from; see tests/golden/make_reference_outputs.py)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_reference_outputs import GEOMETRIES, OUT, SHAPES, shape_spec  # noqa: E402

_cache = {}


def fixture():
    if "f" not in _cache:
        with np.load(OUT) as z:
            _cache["f"] = {k: z[k] for k in z.files}
    return _cache["f"]


def geometry_inputs(name):
    a = fixture()[name + "/inputs"]
    return tuple(np.ascontiguousarray(v) for v in a[:3]), tuple(np.ascontiguousarray(v) for v in a[3:])


def shape_inputs(name):
    return geometry_inputs(name)


def _builder(name):
    mod, fn, kw = GEOMETRIES[name][:3]
    return getattr(__import__(mod, fromlist=[fn]), fn), kw


def product_geometry(name):
    """The product geometry of navigation geometry `name`, closed: replayed from the stored
    builder log (the calls that built the reference's copy) where one is stored, else built
    by its builder."""
    import tempfile

    import vecgeom_gb300 as vg

    if name + "/builder_log" not in fixture():
        fn, kw = _builder(name)
        g = vg.Geometry()
        fn(g, **kw)
        return g
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "g.geom")
        fixture()[name + "/builder_log"].tofile(path)
        g = vg.Geometry.load(path)
    g.close()
    return g


def oracle_geometry(name):
    """The oracle geometry of navigation geometry `name`, made as product_geometry makes it."""
    from oracle.oracle import OracleGeometry
    from oracle.reference import replay_builder_log

    if name + "/builder_log" not in fixture():
        fn, kw = _builder(name)
        o = OracleGeometry()
        fn(o, **kw)
        return o
    return replay_builder_log(fixture()[name + "/builder_log"].tobytes(), OracleGeometry())
