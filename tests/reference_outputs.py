"""Loader of tests/golden/reference_outputs.npz (outputs of the reference's own code; see
tests/golden/make_reference_outputs.py) and the inputs it was made from, regenerated from
the recorded seeds."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_reference_outputs import GEOMETRIES, OUT, SHAPE_POINTS, SHAPE_SEED, SHAPES  # noqa: E402

_cache = {}


def fixture():
    if "f" not in _cache:
        with np.load(OUT) as z:
            _cache["f"] = {k: z[k] for k in z.files}
    return _cache["f"]


def geometry_inputs(name):
    from vecgeom_gb300 import workloads as W

    _, _, _, n, seed, half, _ = GEOMETRIES[name]
    pts, dirs, _ = W.stream_tracks(n, seed, world_half=half)
    return pts, dirs


def shape_inputs(name):
    from vecgeom_gb300 import workloads as W

    lo, hi = fixture()[name + "/box"]
    return W.shape_points_box(lo, hi, SHAPE_POINTS, seed=SHAPE_SEED, scale=1.0)
