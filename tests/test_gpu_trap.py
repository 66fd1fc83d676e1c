"""GPU parity of the trapezoid (UnplacedTrapezoid with its PlaneShell side planes): the six SoA
queries of single trapezoids (the reference unit test's shapes, a general tilted and sheared
one, and that one placed with a rotation) against the oracle, bit-exact, FP64 and mixed; and
the navigator on rings of trapezoids holding corner-built trapezoids: located states and
out-states bit-exact, steps bit-exact, FP64 against the oracle and every mixed schedule
against FP64."""
import numpy as np
import pytest

import golden_util as G
from test_gpu_shapes import edge_points, oracle_all, run_all_queries

pytestmark = pytest.mark.gpu


def trap_specs():
    from vecgeom_gb300 import workloads as W
    doc = G.load("Trap")
    specs = {k: v for k, v in doc["shapes"].items()}
    specs["wedge"] = {"type": "trap", "args": list(W.TRAP_WEDGE)}
    # a long, thin, tilted trapezoid (the parameters of test/unit_tests/TestTrap.cpp TestVECGEOM375)
    deg = np.pi / 180.0
    specs["long"] = {"type": "trap", "args": [1522.0, 1.03516586152568 * deg, -90.4997606158588 * deg, 147.5,
                                              11.0548515319824, 13.62808513641355, 0.4997657953434789 * deg, 92.5,
                                              11.0548515319824, 12.6685743331909, 0.4997660621477440 * deg]}
    return specs


def _compare(got, ref, tag):
    assert np.array_equal(got[0], ref[0]), (tag, "Inside", int((got[0] != ref[0]).sum()))
    assert np.array_equal(got[1], ref[1]), (tag, "Contains", int((got[1] != ref[1]).sum()))
    for q in (2, 3, 4, 5):
        a, b = got[q], ref[q]
        assert np.array_equal(a, b, equal_nan=True), (tag, q, int((a != b).sum()), a[a != b][:4], b[a != b][:4])


@pytest.mark.parametrize("name", sorted(trap_specs()))
def test_trap_queries_bit_exact(cuda, name):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    spec = trap_specs()[name]
    g, o = vg.Geometry(), OracleGeometry()
    pv, opv = G.build(g, spec), G.build(o, spec)
    s = 0
    lo, hi = g.shape_extent(s)
    assert np.array_equal(np.array(o.shape_extent(0)), np.array((lo, hi)))
    inside = lambda x, y, z: o.query(opv, 0, x, y, z)[0]
    dist_out = lambda *a: o.query(opv, 3, *a)[0]
    # a third of the points within 1e-6 mm of the surface, then within 2e-10 mm (inside the
    # 5e-10 mm surface tolerance), then extent-face, integer-rounded and far points
    sets = [W.shape_points_mixed(lo, hi, 3 * 8192, 55, inside, dist_out),
            W.shape_points_mixed(lo, hi, 3 * 8192, 59, inside, dist_out, surface_band=2e-10),
            edge_points(lo, hi, 8192, 56)]
    for k, (pts, dirs) in enumerate(sets):
        ref = oracle_all(o, opv, pts, dirs)
        got = run_all_queries(cuda, g, pv, pts, dirs)
        _compare(got, ref, (name, k, "fp64"))
        mixed = run_all_queries(cuda, g, pv, pts, dirs, flags=vg.PREC_MIXED)
        _compare(mixed, got, (name, k, "mixed"))
        if k == 1:  # all three Inside answers, the surface one included
            assert all((ref[0] == v).sum() > 1000 for v in (1, 2, 3)), np.bincount(ref[0])


def test_trap_placed_with_rotation(cuda):
    """A daughter trapezoid placed with a rotation and translation: the placed-volume queries
    transform points (and directions) to the local frame first, as the oracle's do."""
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    c, s = np.cos(0.7), np.sin(0.7)
    rot = (c, 0.0, s, 0.0, 1.0, 0.0, -s, 0.0, c)  # about y
    tr = (30.0, -20.0, 15.0)
    res = []
    for geo in (vg.Geometry(), OracleGeometry()):
        world_lv = geo.add_logical_volume(geo.add_box(500.0, 500.0, 500.0))
        lv = geo.add_logical_volume(geo.add_trap(*W.TRAP_WEDGE))
        pv = geo.place_daughter(world_lv, lv, tr, rot)
        geo.set_world(geo.place(world_lv))
        geo.close()
        res.append((geo, pv))
    (g, pv), (o, opv) = res
    pts, dirs = W.shape_points_box((-50.0, -90.0, -75.0), (110.0, 70.0, 105.0), 1 << 15, seed=57)
    ref = oracle_all(o, opv, pts, dirs)
    got = run_all_queries(cuda, g, pv, pts, dirs)
    _compare(got, ref, "rotated")
    _compare(run_all_queries(cuda, g, pv, pts, dirs, flags=vg.PREC_MIXED), got, "rotated mixed")
    assert (ref[0] == 1).sum() > 1500


@pytest.fixture(scope="module")
def trap_ring(cuda):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    g, o = vg.Geometry(), OracleGeometry()
    W.build_trap_ring(g)
    W.build_trap_ring(o)
    n = 1 << 16
    gg = np.random.default_rng(58)
    r = 450.0 * np.sqrt(gg.random(n))
    ph = 2 * np.pi * gg.random(n)
    pts = (r * np.cos(ph), r * np.sin(ph), 250.0 * (2 * gg.random(n) - 1))
    dirs = W.isotropic(W.rng(58, 1), n)
    return g, o, pts, dirs


def test_trap_ring_navigation(cuda, trap_ring):
    import vecgeom_gb300 as vg
    from test_gpu_nav import gpu_locate, gpu_step
    g, o, pts, dirs = trap_ring
    st, st_h = gpu_locate(cuda, g, pts)
    ref_st, _ = o.locate(*pts)
    assert np.array_equal(st_h, ref_st)
    out, step, status = gpu_step(cuda, g, pts, dirs, st)
    ref_out, ref_step, _, _ = o.step(*pts, *dirs, ref_st)
    assert (status == 0).all()
    assert np.array_equal(out, ref_out)
    assert np.array_equal(step, ref_step)
    # steps start in the world, the wedges and the inner trapezoids, and cross their faces
    assert len(np.unique(ref_st["nav_ind"])) > 60
    assert (ref_out["nav_ind"] != ref_st["nav_ind"]).mean() > 0.3
    for flags in (vg.PREC_MIXED, vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE):
        o2, s2, e2 = gpu_step(cuda, g, pts, dirs, st, flags=flags)
        assert (e2 == 0).all()
        assert np.array_equal(o2, out), flags
        assert np.array_equal(s2, step), flags
