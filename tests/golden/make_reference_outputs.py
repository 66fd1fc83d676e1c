"""Generate tests/golden/reference_outputs.npz: outputs of the reference's OWN code (its
sources compiled by oracle/build_ref.py against the scalar VecCore stand-in), for the GPU
tests to compare with directly (tests/test_gpu_reference_outputs.py) and the CPU tests to
check the oracle against (tests/test_reference_outputs.py).

Inputs are not stored: they are regenerated from the seeds and boxes recorded here with
vecgeom_gb300.workloads, so the fixture holds only the reference's answers.

* Navigation (GEOMETRIES): the config-5 track starts (stream_tracks(n, seed, world_half)),
  LocateGlobalPoint from the world, then every track transported to the world's edge with
  ComputeStepAndPropagatedState (BVHNavigator): steps per track, final states, and each
  step's next nav index and length (the valid steps of all tracks, concatenated).
* Shapes (SHAPES): the six queries of each config-1 and config-2 shape (unplaced, the shape's
  own frame) on points uniform in the recorded box (its 1.2x extent) with isotropic directions.

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
SHAPES = ["box", "tube", "cone", "tube_phi", "polycone", "polyhedron", "torus2", "trd", "box_minus_tube"]
SHAPE_POINTS = 256
SHAPE_SEED = 0x5A


def main():
    from oracle import reference as R
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W

    out = {}
    for name, (mod, fn, kw, n, seed, half, max_steps) in GEOMETRIES.items():
        (x, y, z), (dx, dy, dz), _ = W.stream_tracks(n, seed, world_half=half)
        st, (ns, final, tr, trs, _) = R.run((mod, fn), [("locate_transport", (x, y, z, dx, dy, dz, max_steps), {})],
                                            kw)[0]
        mask = np.arange(max_steps)[None, :] < ns[:, None]
        out[name + "/start"] = st.view(np.uint8).reshape(n, 12)
        out[name + "/nsteps"] = ns.astype(np.int32)
        out[name + "/final"] = final.view(np.uint8).reshape(n, 12)
        out[name + "/trace_nav"] = tr[mask].astype(np.uint32)
        out[name + "/trace_step"] = trs[mask]
    shapes = [W.SHAPES_CFG1.get(s) or W.SHAPES_CFG2[s] for s in SHAPES]
    o = OracleGeometry()
    ids = [W.add_shape(o, k, p) for k, p in shapes]
    calls, keys = [], []
    for name, sid in zip(SHAPES, ids):
        lo, hi = o.shape_extent(sid)
        c, h = 0.5 * (lo + hi), 0.6 * (hi - lo)  # the 1.2x extent box
        out[name + "/box"] = np.stack([c - h, c + h])
        pts, dirs = W.shape_points_box(c - h, c + h, SHAPE_POINTS, seed=SHAPE_SEED, scale=1.0)
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
