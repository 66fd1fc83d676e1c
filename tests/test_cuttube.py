"""Cut tube on the CPU: the oracle's restatement of UnplacedCutTube against the Tube (pinned by
the TestTube known answers): with flat cut planes a cut tube is that tube, so Inside,
Contains and safeties are bit-identical and distances agree within 1e-9 mm away from the
z faces' tolerance bands (the cut planes' surface band is kTolerance, the tube's z band
kHalfTolerance; for points outside DistanceToOut gives the planes' -kInfLength where the
tube gives -1); the product's builder gives the oracle's extents, including the phi
reductions of UnplacedCutTube::Extent, and rejects the normals the reference rejects."""
import numpy as np
import pytest

import vecgeom_gb300 as vg
from conftest import dist_mismatch
from oracle.oracle import OracleGeometry
from test_cpu_build import HostOnly
from vecgeom_gb300 import workloads as W

CUTS = [
    (0.0, 20.0, 30.0, 0.0, 2 * np.pi, (0.0, 0.0, -1.0), (0.0, 0.0, 1.0)),
    (5.0, 20.0, 30.0, 0.5, 1.7, (0.0, -0.7, -0.71), (0.7, 0.0, 0.71)),
    (10.0, 20.0, 30.0, 0.0, 4.0, (0.2, 0.3, -1.0), (-0.1, 0.5, 1.0)),
    (0.0, 50.0, 10.0, 2.0, 5.0, (-15.0, -15.0, -15.0), (10.0, 10.0, 10.0)),
]


def _pv(o, shape):
    return o.place(o.add_logical_volume(shape))


def test_flat_cut_tube_is_the_tube():
    o = OracleGeometry()
    rmin, rmax, dz, sphi, dphi, b, t = CUTS[0]
    ct = _pv(o, o.add_cut_tube(rmin, rmax, dz, sphi, dphi, b, t))
    tb = _pv(o, o.add_tube(rmin, rmax, dz, sphi, dphi))
    o.close()
    (x, y, z), dirs = W.shape_points_box((-rmax, -rmax, -dz), (rmax, rmax, dz), 1 << 16, 77)
    keep = np.abs(np.abs(z) - dz) > 1e-6
    x, y, z = x[keep], y[keep], z[keep]
    dirs = [d[keep] for d in dirs]
    for q in (0, 1, 4, 5):
        assert np.array_equal(o.query(ct, q, x, y, z)[0], o.query(tb, q, x, y, z)[0]), q
    for q in (2, 3):
        a = o.query(ct, q, x, y, z, *dirs)[0]
        b_ = o.query(tb, q, x, y, z, *dirs)[0]
        if q == 3:
            # outside points: the tube's DistanceToOut gives -1, the cut planes' -kInfLength
            # (Plane::DistanceToOut, Plane.h:149-170), both the reference's outside answers
            out = b_ == -1.0
            assert (a[out] < 0).all()
            a, b_ = a[~out], b_[~out]
        assert not dist_mismatch(a, b_).any(), (q, int(dist_mismatch(a, b_).sum()))


@pytest.mark.parametrize("k", range(len(CUTS)))
def test_extents_match_oracle(k):
    p, o = vg.Geometry(), OracleGeometry()
    sp = p.add_cut_tube(*CUTS[k])
    so = o.add_cut_tube(*CUTS[k])
    lo_p, hi_p = p.shape_extent(sp)
    lo_o, hi_o = o.shape_extent(so)
    assert np.array_equal(lo_p, lo_o) and np.array_equal(hi_p, hi_o)
    pv = _pv(o, so)
    o.close()
    (x, y, z), _ = W.shape_points_box(lo_o, hi_o, 1 << 14, 5 + k, scale=1.0)
    assert o.query(pv, 1, x, y, z)[0].astype(bool).any()


def test_illegal_normals_rejected():
    g = vg.Geometry()
    with pytest.raises(vg.VGError, match="normal"):
        g.add_cut_tube(0.0, 10.0, 5.0, 0.0, 2 * np.pi, (0.0, 0.0, 1.0), (0.0, 0.0, 1.0))
    with pytest.raises(vg.VGError, match="normal"):
        g.add_cut_tube(0.0, 10.0, 5.0, 0.0, 2 * np.pi, (0.0, 0.0, -1.0), (0.3, 0.0, -0.1))


def test_cut_tube_geometry_builds_identically():
    p, o = vg.Geometry(), OracleGeometry()
    W.build_cut_tube_ring(HostOnly(p))
    W.build_cut_tube_ring(o)
    assert np.array_equal(p.nav_table(), o.nav_table())
    assert o.check_nav_index(p.nav_table())[0] == 0
