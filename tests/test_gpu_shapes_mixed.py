"""Mixed-precision shape queries (VG_PREC_MIXED on the placed SoA queries) against the FP64
kernels on the same points: Inside, Contains, DistanceToIn and DistanceToOut are identical
for every shape; safeties are identical except the full-phi Tube's, whose FP32 safeties
never exceed the FP64 value and stay within the stated bound 2^-20 (max(r, |z|) +
max(dz, rmax)) below it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
QUERIES = ["inside", "contains", "distance_to_in", "distance_to_out", "safety_to_in", "safety_to_out"]


def _run(torch, g, pv, pts, dirs, flags):
    t = [torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (*pts, *dirs)]
    n = len(pts[0])
    res = {}
    for q in QUERIES:
        dt = torch.int32 if q == "inside" else (torch.uint8 if q == "contains" else torch.float64)
        o = torch.empty(n, dtype=dt, device="cuda:0")
        fn = getattr(g, q)
        if q.startswith("distance"):
            fn(pv, *t, o, flags=flags)
        else:
            fn(pv, *t[:3], o, flags=flags)
        res[q] = o.cpu().numpy()
    return res


def _cases():
    from vecgeom_gb300 import workloads as W
    c = [(k, v) for k, v in W.SHAPES_CFG1.items()] + [(k, v) for k, v in W.SHAPES_CFG2.items()]
    c.append(("polyhedron_phi", ("polyhedron", (0.3, 1.8, 5, (-100.0, 0.0, 0.0, 50.0), (0.0, 10.0, 20.0, 5.0),
                                                (40.0, 60.0, 50.0, 30.0)))))
    return c


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
def test_mixed_shape_queries(cuda, case):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    name, (kind, params) = case
    g = vg.Geometry()
    s, pv = W.build_single_shape(g, kind, params)
    lo, hi = g.shape_extent(s)
    inside = lambda x, y, z: _run(cuda, g, pv, (x, y, z), (x, y, z), vg.PREC_FP64)["inside"]

    def dout(x, y, z, dx, dy, dz):
        return _run(cuda, g, pv, (x, y, z), (dx, dy, dz), vg.PREC_FP64)["distance_to_out"]

    pts, dirs = W.shape_points_mixed(lo, hi, 3 * 8192, 123, inside, dout)
    a = _run(cuda, g, pv, pts, dirs, vg.PREC_FP64)
    b = _run(cuda, g, pv, pts, dirs, vg.PREC_MIXED)
    for q in QUERIES[:4]:
        assert np.array_equal(a[q], b[q]), (q, int((a[q] != b[q]).sum()))
    if kind == "tube" and params[4] >= 2 * np.pi:
        r = np.hypot(pts[0], pts[1])
        bound = 2.0 ** -20 * (np.maximum(r, np.abs(pts[2])) + max(params[1], params[2]))
        for q in ("safety_to_in", "safety_to_out"):
            assert (b[q] <= a[q]).all(), q
            assert (a[q] - b[q] <= bound * 1.0001 + 1e-300).all(), q
            assert (a[q] != b[q]).any(), q  # the FP32 form ran
    else:
        for q in ("safety_to_in", "safety_to_out"):
            assert np.array_equal(a[q], b[q]), q


def test_mixed_placed_transform(cuda):
    """A rotated and translated tube: the FP32 guard works in the local frame."""
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    g = vg.Geometry()
    lv = g.add_logical_volume(g.add_tube(10.0, 20.0, 30.0, 0.3, 1.8))
    pv = g.place(lv, (5.0, -7.0, 11.0), W.rot_z(0.7))
    g.close()
    (x, y, z), dirs = W.shape_points_box((-30.0, -35.0, -25.0), (40.0, 25.0, 45.0), 1 << 16, 9)
    a = _run(cuda, g, pv, (x, y, z), dirs, vg.PREC_FP64)
    b = _run(cuda, g, pv, (x, y, z), dirs, vg.PREC_MIXED)
    for q in QUERIES:
        assert np.array_equal(a[q], b[q]), q


# Polyhedra for the FP32-screened distances: the config-2 one, phi cut-outs below and above
# pi, inner radii on some segments, and a z plane shared by two segments (the same-z case of
# Quadrilaterals::DistanceToOut).
POLYHEDRA = [
    (0.3, 1.8, 5, (-100.0, 0.0, 0.0, 50.0), (0.0, 10.0, 20.0, 5.0), (40.0, 60.0, 50.0, 30.0)),
    (0.0, 4.5, 3, (-10.0, 10.0), (0.0, 0.0), (20.0, 30.0)),
    (0.5, 2 * np.pi, 6, (-50.0, -20.0, 30.0, 60.0), (10.0, 0.0, 0.0, 15.0), (40.0, 45.0, 45.0, 20.0)),
    (0.0, 2 * np.pi, 8, (-300.0, -100.0, -100.0, 200.0, 400.0), (50.0, 60.0, 80.0, 80.0, 0.0),
     (150.0, 200.0, 250.0, 300.0, 100.0)),
]


@pytest.mark.parametrize("k", range(len(POLYHEDRA)))
def test_mixed_polyhedron_distances_equal_fp64(cuda, k):
    """Near-surface, inside and outside points; a third of the rays along the axes or in the
    xy plane (grazing the side faces, parallel to the z planes), where the FP32 screen must
    leave every quadrilateral to FP64."""
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    g = vg.Geometry()
    s, pv = W.build_single_shape(g, "polyhedron", POLYHEDRA[k])
    lo, hi = g.shape_extent(s)
    inside = lambda x, y, z: _run(cuda, g, pv, (x, y, z), (x, y, z), vg.PREC_FP64)["inside"]

    def dout(x, y, z, dx, dy, dz):
        return _run(cuda, g, pv, (x, y, z), (dx, dy, dz), vg.PREC_FP64)["distance_to_out"]

    pts, dirs = W.shape_points_mixed(lo, hi, 3 * 16384, 321 + k, inside, dout)
    n = len(pts[0])
    dirs = [np.array(c) for c in dirs]
    rng = np.random.default_rng(k)
    sel = rng.random(n) < 1 / 3
    axis = rng.integers(0, 8, n)
    for i in np.flatnonzero(sel):
        a = axis[i]
        if a < 6:
            v = [0.0, 0.0, 0.0]
            v[a // 2] = 1.0 if a % 2 == 0 else -1.0
        else:
            ph = rng.random() * 2 * np.pi
            v = [np.cos(ph), np.sin(ph), 0.0]
        for c in range(3):
            dirs[c][i] = v[c]
    a = _run(cuda, g, pv, pts, dirs, vg.PREC_FP64)
    b = _run(cuda, g, pv, pts, dirs, vg.PREC_MIXED)
    for q in ("distance_to_in", "distance_to_out"):
        assert np.array_equal(a[q].view(np.int64), b[q].view(np.int64)), (q, int((a[q] != b[q]).sum()))


POLYCONES = [
    (0.0, 2 * np.pi, (-500.0, -300.0, -100.0, 0.0, 250.0, 500.0), (50.0, 60.0, 0.0, 0.0, 80.0, 120.0),
     (150.0, 300.0, 200.0, 400.0, 380.0, 390.0)),
    (0.4, 2.5, (-40.0, -10.0, 10.0, 40.0), (5.0, 10.0, 10.0, 2.0), (20.0, 30.0, 25.0, 50.0)),
    (0.0, 2 * np.pi, (-1.0, 0.0, 1.0, 300.0), (0.0, 0.0, 0.0, 0.0), (100.0, 10.0, 300.0, 5.0)),
]


@pytest.mark.parametrize("k", range(len(POLYCONES)))
def test_mixed_polycone_distances_equal_fp64(cuda, k):
    """Polycones with hollow, solid, steep and phi-cut sections: the FP32 section screen of
    DistanceToIn gives the FP64 results bit for bit, also for rays along the axes."""
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    g = vg.Geometry()
    s, pv = W.build_single_shape(g, "polycone", POLYCONES[k])
    lo, hi = g.shape_extent(s)
    inside = lambda x, y, z: _run(cuda, g, pv, (x, y, z), (x, y, z), vg.PREC_FP64)["inside"]

    def dout(x, y, z, dx, dy, dz):
        return _run(cuda, g, pv, (x, y, z), (dx, dy, dz), vg.PREC_FP64)["distance_to_out"]

    pts, dirs = W.shape_points_mixed(lo, hi, 3 * 16384, 555 + k, inside, dout)
    dirs = [np.array(c) for c in dirs]
    rng = np.random.default_rng(50 + k)
    sel = np.flatnonzero(rng.random(len(pts[0])) < 0.25)
    for i in sel:
        a = rng.integers(0, 6)
        for c in range(3):
            dirs[c][i] = (1.0 if a % 2 == 0 else -1.0) if c == a // 2 else 0.0
    a = _run(cuda, g, pv, pts, dirs, vg.PREC_FP64)
    b = _run(cuda, g, pv, pts, dirs, vg.PREC_MIXED)
    for q in ("distance_to_in", "distance_to_out"):
        assert np.array_equal(a[q].view(np.int64), b[q].view(np.int64)), (q, int((a[q] != b[q]).sum()))
