"""Generate tests/golden/reference_outputs.npz: outputs of the reference's OWN code (its
sources compiled by oracle/build_ref.py against the scalar VecCore stand-in), for the GPU
tests to compare with directly (tests/test_gpu_reference_outputs.py) and the CPU tests to
check the oracle against (tests/test_reference_outputs.py).

The inputs are stored with the answers: the track directions pass through numpy's
transcendental functions, whose last bit can differ between machines (x86-64 here, aarch64
on the GPU machine), which would move the steps by ulps. For the same reason the GDML
detector is stored as the product's builder log (vg_geom_save) of the calls that built the
reference's copy: the GDML reader's angle conversions go through the C library. The barrel
and the detector are rebuilt by their builders (their rotations are identical on both
machines, and the detector's log would be megabytes).

* Navigation (GEOMETRIES): the config-5 track starts (stream_tracks(n, seed, world_half)),
  LocateGlobalPoint from the world, then every track transported to the world's edge with
  ComputeStepAndPropagatedState (BVHNavigator): steps per track, final states, and each
  step's next nav index and length (the valid steps of all tracks, concatenated).
* Shapes (SHAPES): the six queries of each config-1 and config-2 shape and of a Polyhedron
  with a phi cut, a Trapezoid, two Spheres, two Hypes, a CutTube and two twisted GenTraps
  (unplaced, the shape's own frame) on points uniform in the 1.2x extent box with isotropic
  directions.

Run here, where the reference tree is present:  python tests/golden/make_reference_outputs.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "reference_outputs.npz")
WL = "vecgeom_gb300.workloads"
GDML = os.path.join(HERE, "gdml", "detector.gdml")
# name: (builder module, builder, builder kwargs, tracks, seed, world half-lengths, max steps)
GEOMETRIES = {
    "barrel": (WL, "build_barrel", {}, 256, 0xB1, (2000.0, 2000.0, 3000.0), 1000),
    "detector": (WL, "build_detector", {}, 256, 0xD2, (2000.0, 2000.0, 3000.0), 1000),
    "gdml_detector": ("oracle.reference", "build_gdml", {"path": GDML}, 256, 0xD3, (1500.0, 1500.0, 2000.0), 1000),
}
STORED_GEOMETRIES = ("gdml_detector",)
SHAPES = ["box", "tube", "cone", "tube_phi", "polycone", "polyhedron", "torus2", "trd", "box_minus_tube",
          "polyhedron_phi", "trap_wedge", "sphere_phi", "sphere_theta", "hype_hollow", "hype_cone_in", "cut_tube",
          "gentrap_twisted", "gentrap_one_twisted"]
_PI = 3.141592653589793
# the shapes beyond configs 1-2: (kind, parameters) as vecgeom_gb300.workloads.add_shape takes them
EXTRA_SHAPES = {
    "polyhedron_phi": ("polyhedron", (0.3, 1.8, 5, (-100.0, 0.0, 0.0, 50.0), (0.0, 10.0, 20.0, 5.0),
                                      (40.0, 60.0, 50.0, 30.0))),
    "trap_wedge": ("trap", (60.0, 0.1, 0.4, 40.0, 20.0, 30.0, 0.15, 50.0, 25.0, 35.0, 0.15)),
    "sphere_phi": ("sphere", (20.0, 50.0, 0.3, 1.8, 0.0, _PI)),
    "sphere_theta": ("sphere", (10.0, 50.0, 0.5, 2.5, 1.8, 0.9)),
    "cut_tube": ("cut_tube", (10.0, 20.0, 30.0, 0.0, 4.0, (0.2, 0.3, -1.0), (-0.1, 0.5, 1.0))),
}


def shape_spec(name):
    from vecgeom_gb300 import workloads as W

    if name.startswith("hype_"):
        return ("hype", W.HYPES[name[5:]])
    if name.startswith("gentrap_"):
        return ("gentrap", W.GENTRAPS[name[8:]])
    return EXTRA_SHAPES.get(name) or W.SHAPES_CFG1.get(name) or W.SHAPES_CFG2[name]
SHAPE_POINTS = 256
SHAPE_SEED = 0x5A


class _Open:
    """A product geometry whose close() is skipped: only the builder log is wanted."""

    def __init__(self, g):
        self.g = g

    def __getattr__(self, n):
        return getattr(self.g, n)

    def close(self):
        pass


def main():
    from oracle import reference as R
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W

    import tempfile

    import vecgeom_gb300 as vg

    out = {}
    for name, (mod, fn, kw, n, seed, half, max_steps) in GEOMETRIES.items():
        if name in STORED_GEOMETRIES:
            p = vg.Geometry()
            getattr(__import__(mod, fromlist=[fn]), fn)(_Open(p), **kw)
            with tempfile.TemporaryDirectory() as d:
                p.save(os.path.join(d, "g.geom"))
                with open(os.path.join(d, "g.geom"), "rb") as fh:
                    out[name + "/builder_log"] = np.frombuffer(fh.read(), dtype=np.uint8)
        (x, y, z), (dx, dy, dz), _ = W.stream_tracks(n, seed, world_half=half)
        st, (ns, final, tr, trs, _) = R.run((mod, fn), [("locate_transport", (x, y, z, dx, dy, dz, max_steps), {})],
                                            kw)[0]
        mask = np.arange(max_steps)[None, :] < ns[:, None]
        out[name + "/inputs"] = np.stack([x, y, z, dx, dy, dz])
        out[name + "/start"] = st.view(np.uint8).reshape(n, 12)
        out[name + "/nsteps"] = ns.astype(np.int32)
        out[name + "/final"] = final.view(np.uint8).reshape(n, 12)
        out[name + "/trace_nav"] = tr[mask].astype(np.uint32)
        out[name + "/trace_step"] = trs[mask]
    shapes = [shape_spec(s) for s in SHAPES]
    o = OracleGeometry()
    ids = [W.add_shape(o, k, p) for k, p in shapes]
    calls, keys = [], []
    for name, sid in zip(SHAPES, ids):
        lo, hi = o.shape_extent(sid)
        c, h = 0.5 * (lo + hi), 0.6 * (hi - lo)  # the 1.2x extent box
        out[name + "/box"] = np.stack([c - h, c + h])
        pts, dirs = W.shape_points_box(c - h, c + h, SHAPE_POINTS, seed=SHAPE_SEED, scale=1.0)
        out[name + "/inputs"] = np.stack([*pts, *dirs])
        for q in range(6):
            d = dirs if q in (2, 3) else (None, None, None)
            calls.append(("shape_query", (sid, q, *pts, *d), {}))
            keys.append("%s/q%d" % (name, q))
    got = R.run(("oracle.reference", "build_shapes"), calls, {"shapes": shapes})
    for k, v in zip(keys, got):
        out[k] = np.asarray(v)
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
