"""The CUDA path against outputs of the reference's OWN code (tests/golden/reference_outputs.npz,
made by tests/golden/make_reference_outputs.py from the reference's sources compiled here
against the VecCore stand-in; tests/test_reference_outputs.py checks the oracle against the
same fixture on the CPU):

* LocateGlobalPoint and whole transport histories (vg_nav_transport, plain FP64 and the mixed
  + sorted + work-queue schedule) in the barrel, the config-4 detector and the GDML detector
  (replayed from the stored builder log of the reference's copy): steps per track, final
  states, every step's next nav index and length, bit for bit, except the steps into or out
  of the GDML detector's Torus2 ring (within 1e-9 mm + 1e-12 relative: the device's
  cbrt/pow/cos/atan2);
* the six unplaced queries of 18 shapes (configs 1-2, a phi-cut Polyhedron, a Trapezoid,
  two Spheres, two Hypes, a CutTube, two twisted GenTraps), FP64 and mixed precision:
  bit for bit, except Torus2's distances (within 1e-9 mm + 1e-12 relative: its cubic
  resolvent calls the device's cbrt/pow/cos/atan2) and the full-phi Tube's mixed-precision
  safeties (the stated FP32 bound)."""
import numpy as np
import pytest

from reference_outputs import GEOMETRIES, SHAPES, fixture, geometry_inputs, shape_spec, oracle_geometry, product_geometry, shape_inputs

pytestmark = pytest.mark.gpu

QUERIES = ["inside", "contains", "distance_to_in", "distance_to_out", "safety_to_in", "safety_to_out"]


@pytest.mark.parametrize("name", sorted(GEOMETRIES))
def test_transport_equals_reference_outputs(cuda, name):
    import vecgeom_gb300 as vg
    f = fixture()
    n, max_steps = GEOMETRIES[name][3], GEOMETRIES[name][6]
    g = product_geometry(name)  # the builder calls of the reference's copy, replayed
    pts, dirs = geometry_inputs(name)
    mask = np.arange(max_steps)[None, :] < f[name + "/nsteps"][:, None]
    for flags in (vg.PREC_FP64, vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE):
        dev = [cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (*pts, *dirs)]
        st = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
        g.locate_point(*dev[:3], st)
        assert np.array_equal(st.cpu().numpy().reshape(n, 12), f[name + "/start"])
        nsteps, status, _, tst, tsp = g.transport(*dev, st, max_steps=max_steps, flags=flags, trace_tracks=n)
        assert (status.cpu().numpy() == 0).all()
        assert np.array_equal(nsteps.cpu().numpy(), f[name + "/nsteps"]), flags
        assert np.array_equal(st.cpu().numpy().reshape(n, 12), f[name + "/final"]), flags
        trs = tst.cpu().numpy().view(vg.NAVSTATE_DTYPE).reshape(n, max_steps)["nav_ind"]
        tsl = tsp.cpu().numpy().reshape(n, max_steps)
        assert np.array_equal(trs[mask], f[name + "/trace_nav"]), flags
        got, ref = tsl[mask], f[name + "/trace_step"]
        if name != "gdml_detector":
            assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), flags
            continue
        # the GDML detector holds a Torus2 ring: steps into or out of it are compared at
        # 1e-9 mm + 1e-12 relative (the device's cbrt/pow/cos/atan2), every other step bit
        # for bit
        torus = oracle_geometry(name).locate(np.array([1000.0]), np.array([0.0]), np.array([1500.0]))[0]["nav_ind"][0]
        nav = f[name + "/trace_nav"]
        first = np.concatenate([[0], np.cumsum(f[name + "/nsteps"])[:-1]])
        prev = np.concatenate([[0], nav[:-1]])
        moved = f[name + "/nsteps"] > 0
        prev[first[moved]] = f[name + "/start"].reshape(-1).view(vg.NAVSTATE_DTYPE)["nav_ind"][moved]
        differ = got != ref
        assert (np.abs(got - ref)[differ] <= 1e-9 + 1e-12 * np.abs(ref[differ])).all(), flags
        assert ((nav == torus) | (prev == torus))[differ].all(), flags
        assert differ.sum() < 0.02 * got.size, flags


@pytest.mark.parametrize("name", SHAPES)
def test_shape_queries_equal_reference_outputs(cuda, name):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    f = fixture()
    g = vg.Geometry()
    s, _ = W.build_single_shape(g, *shape_spec(name))
    pts, dirs = shape_inputs(name)
    t = [cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (*pts, *dirs)]
    n = len(pts[0])
    for flags in (vg.PREC_FP64, vg.PREC_MIXED):
        for qi, q in enumerate(QUERIES):
            dt = {0: cuda.int32, 1: cuda.uint8}.get(qi, cuda.float64)
            out = cuda.empty(n, dtype=dt, device="cuda:0")
            if qi in (2, 3):
                g.shape_query(q, s, *t[:3], out, *t[3:], flags=flags)
            else:
                g.shape_query(q, s, *t[:3], out, flags=flags)
            got = out.cpu().numpy()
            ref = f["%s/q%d" % (name, qi)]
            if qi < 2:
                assert np.array_equal(got.astype(np.int32), ref.astype(np.int32)), (q, flags)
            elif name == "torus2" and qi in (2, 3):  # device cbrt/pow/cos/atan2 in the resolvent
                bad = ~((got == ref) | (np.abs(got - ref) <= 1e-9 + 1e-12 * np.abs(ref)))
                assert not bad.any(), (q, flags, int(bad.sum()))
            elif name == "tube" and qi in (4, 5) and flags == vg.PREC_MIXED:
                # full-phi Tube, FP32 safeties: never above FP64, at most the stated bound below
                _, params = W.SHAPES_CFG1["tube"]
                bound = 2.0 ** -20 * (np.maximum(np.hypot(pts[0], pts[1]), np.abs(pts[2])) + max(params[1], params[2]))
                assert (got <= ref).all() and (ref - got <= bound * 1.0001 + 1e-300).all(), (q, flags)
            else:
                assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), (q, flags)
