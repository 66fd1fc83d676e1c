"""GPU parity of the FP64 SoA shape queries against the oracle (config-1 shapes and
points; extra edge-case points on every surface, axis-aligned directions, far points).

Bar: Inside/Contains bit-exact; distances and safeties within 1e-9 mm + 1e-12 relative,
with kInfLength and -1 sentinels matching exactly."""
import numpy as np
import pytest

from conftest import dist_mismatch

pytestmark = pytest.mark.gpu

N = 1 << 16


def run_all_queries(torch, g, pv, pts, dirs, flags=0):
    dev = torch.device("cuda:0")
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (*pts, *dirs)]
    n = len(pts[0])
    res = {}
    o_i = torch.empty(n, dtype=torch.int32, device=dev)
    g.inside(pv, t[0], t[1], t[2], o_i, flags)
    res[0] = o_i.cpu().numpy()
    o_b = torch.empty(n, dtype=torch.uint8, device=dev)
    g.contains(pv, t[0], t[1], t[2], o_b, flags)
    res[1] = o_b.cpu().numpy().astype(np.int32)
    for q, fn in ((2, g.distance_to_in), (3, g.distance_to_out)):
        o = torch.empty(n, dtype=torch.float64, device=dev)
        fn(pv, *t, o, flags=flags)
        res[q] = o.cpu().numpy()
    for q, fn in ((4, g.safety_to_in), (5, g.safety_to_out)):
        o = torch.empty(n, dtype=torch.float64, device=dev)
        fn(pv, t[0], t[1], t[2], o, flags)
        res[q] = o.cpu().numpy()
    return res


def oracle_all(o, pv, pts, dirs):
    return {q: o.query(pv, q, *pts, *dirs)[0] for q in range(6)}


def edge_points(lo, hi, n, seed):
    """Points on the extent faces, edges and at far distance, with axis-aligned and
    random directions."""
    g = np.random.default_rng(seed)
    lo, hi = np.asarray(lo), np.asarray(hi)
    pts = np.empty((n, 3))
    k = n // 4
    pts[:k] = lo + (hi - lo) * g.random((k, 3))
    face = g.integers(0, 3, k)
    pts[:k][np.arange(k), face] = np.where(g.random(k) < 0.5, lo[face], hi[face])
    pts[k:2 * k] = np.round(lo + (hi - lo) * g.random((k, 3)))
    pts[2 * k:3 * k] = 1e4 * (2 * g.random((k, 3)) - 1)
    pts[3 * k:] = 0.5 * (lo + hi) + 0.01 * (2 * g.random((n - 3 * k, 3)) - 1)
    axes = np.eye(3)[g.integers(0, 3, n)] * np.where(g.random((n, 1)) < 0.5, -1.0, 1.0)
    d = g.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    d[: n // 2] = axes[: n // 2]
    return tuple(pts.T.copy()), tuple(d.T.copy())


@pytest.mark.parametrize("name", ["box", "tube", "cone"])
def test_cfg1_shape_parity(cuda, name):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    from oracle.oracle import OracleGeometry

    kind, params = W.SHAPES_CFG1[name]
    g, o = vg.Geometry(), OracleGeometry()
    s, pv = W.build_single_shape(g, kind, params)
    W.build_single_shape(o, kind, params)
    lo, hi = g.shape_extent(s)
    for pts, dirs in (W.shape_points_box(lo, hi, N, seed=1234), edge_points(lo, hi, 8192, 99)):
        got = run_all_queries(cuda, g, pv, pts, dirs)
        ref = oracle_all(o, pv, pts, dirs)
        assert np.array_equal(got[0], ref[0]), "Inside"
        assert np.array_equal(got[1], ref[1]), "Contains"
        for q in (2, 3, 4, 5):
            bad = dist_mismatch(got[q], ref[q])
            assert not bad.any(), (q, int(bad.sum()), got[q][bad][:4], ref[q][bad][:4])


def test_tube_and_cone_variants_parity(cuda):
    """Hollow, sectioned and tapered variants (phi < pi, phi > pi, rmin = 0)."""
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W

    variants = [("tube", (0.0, 50.0, 50.0, 0.0, 0.5 * np.pi)), ("tube", (45.0, 50.0, 50.0, 0.5 * np.pi, 1.5 * np.pi)),
                ("tube", (750.0, 760.0, 350.0, 0.31415926535897931, 5.6548667764616276)),
                ("cone", (0.0, 50.0, 0.0, 100.0, 50.0, 0.0, 2 * np.pi)),
                ("cone", (10.0, 20.0, 30.0, 40.0, 25.0, 0.3, 1.2)),
                ("cone", (10.0, 20.0, 10.0, 20.0, 25.0, 1.0, 4.0))]
    for kind, params in variants:
        g, o = vg.Geometry(), OracleGeometry()
        s, pv = W.build_single_shape(g, kind, params)
        W.build_single_shape(o, kind, params)
        lo, hi = g.shape_extent(s)
        pts, dirs = W.shape_points_box(lo, hi, 16384, seed=5)
        got = run_all_queries(cuda, g, pv, pts, dirs)
        ref = oracle_all(o, pv, pts, dirs)
        assert np.array_equal(got[0], ref[0]), (kind, params)
        for q in (2, 3, 4, 5):
            assert not dist_mismatch(got[q], ref[q]).any(), (kind, params, q)


def test_placed_transform_parity(cuda):
    """A rotated, translated placement: the mother-frame queries transform first."""
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W

    rot = W.rot_z(0.7)
    for geo in (vg.Geometry(), OracleGeometry()):
        lv = geo.add_logical_volume(geo.add_cone(5.0, 10.0, 8.0, 15.0, 25.0, 0.0, 2 * np.pi))
        geo.place(lv, (3.0, -4.0, 5.0), rot)
        geo.close()
        if isinstance(geo, vg.Geometry):
            g = geo
        else:
            o = geo
    pts, dirs = W.shape_points_box((-20, -20, -30), (20, 20, 30), 16384, seed=8)
    got = run_all_queries(cuda, g, 0, pts, dirs)
    ref = oracle_all(o, 0, pts, dirs)
    assert np.array_equal(got[0], ref[0])
    for q in (2, 3, 4, 5):
        assert not dist_mismatch(got[q], ref[q]).any(), q


# Every shape meets 1e-9 mm + 1e-12 relative against the FP64 oracle. Torus2 is the one
# shape whose results are not all bit-identical: its cubic resolvent calls cbrt/pow/cos/atan2,
# whose CUDA and libm results differ in the last ulps, and the Newton polish then stops
# within kTolerance of the root (measured on 2^22 config-2 points: at most 9.6e-10 mm for
# DistanceToIn and 5.5e-10 mm for DistanceToOut; Inside and the safeties bit-identical).
CFG2_TOL = {}


@pytest.mark.parametrize("name", ["tube_phi", "polycone", "polyhedron", "torus2", "trd", "box_minus_tube"])
def test_cfg2_shape_parity(cuda, name):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W

    kind, params = W.SHAPES_CFG2[name]
    g, o = vg.Geometry(), OracleGeometry()
    s, pv = W.build_single_shape(g, kind, params)
    W.build_single_shape(o, kind, params)
    lo, hi = g.shape_extent(s)
    pts, dirs = W.shape_points_mixed(lo, hi, 3 * 8192, 77, lambda x, y, z: o.query(pv, 0, x, y, z)[0],
                                     lambda *a: o.query(pv, 3, *a)[0])
    got = run_all_queries(cuda, g, pv, pts, dirs)
    ref = oracle_all(o, pv, pts, dirs)
    tol = CFG2_TOL.get(name, 1e-9)
    assert np.array_equal(got[0], ref[0]), ("Inside", int((got[0] != ref[0]).sum()))
    assert np.array_equal(got[1], ref[1]), ("Contains", int((got[1] != ref[1]).sum()))
    for q in (2, 3, 4, 5):
        bad = dist_mismatch(got[q], ref[q], abs_tol=tol)
        assert not bad.any(), (q, int(bad.sum()), got[q][bad][:4], ref[q][bad][:4])


# Polyhedron variants beyond the config-2 shape: phi cut-outs smaller and larger than pi,
# a z plane shared by two segments (the border case), inner radii on some segments only.
POLYHEDRA = [
    (0.3, 1.8, 5, (-100.0, 0.0, 0.0, 50.0), (0.0, 10.0, 20.0, 5.0), (40.0, 60.0, 50.0, 30.0)),
    (0.0, 4.5, 3, (-10.0, 10.0), (0.0, 0.0), (20.0, 30.0)),
    (0.5, 2 * np.pi, 6, (-50.0, -20.0, 30.0, 60.0), (10.0, 0.0, 0.0, 15.0), (40.0, 45.0, 45.0, 20.0)),
]


@pytest.mark.parametrize("k", range(len(POLYHEDRA)))
def test_polyhedron_variants_parity(cuda, k):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    g, o = vg.Geometry(), OracleGeometry()
    s, pv = W.build_single_shape(g, "polyhedron", POLYHEDRA[k])
    W.build_single_shape(o, "polyhedron", POLYHEDRA[k])
    lo, hi = g.shape_extent(s)
    pts, dirs = W.shape_points_mixed(lo, hi, 3 * 4096, 91 + k, lambda x, y, z: o.query(pv, 0, x, y, z)[0],
                                     lambda *a: o.query(pv, 3, *a)[0])
    got = run_all_queries(cuda, g, pv, pts, dirs)
    ref = oracle_all(o, pv, pts, dirs)
    assert np.array_equal(got[0], ref[0]), ("Inside", int((got[0] != ref[0]).sum()))
    assert np.array_equal(got[1], ref[1]), ("Contains", int((got[1] != ref[1]).sum()))
    for q in (2, 3, 4, 5):
        bad = dist_mismatch(got[q], ref[q])
        assert not bad.any(), (q, int(bad.sum()), got[q][bad][:4], ref[q][bad][:4])
