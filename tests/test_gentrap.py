"""GenTrap on the CPU: the product's builder accepts exactly the vertex sets the reference's
GenTrapStruct::Initialize accepts (clockwise or anticlockwise bases, degenerated edges and
collapsed bases) and rejects the ones it reports as errors (opposite orientations, crossing
opposite segments, non-convex bases, dz <= 0); an anticlockwise GenTrap answers every query
as its clockwise reordering does; the GenTrap ring builds identically in the product and the
oracle."""
import numpy as np
import pytest

import vecgeom_gb300 as vg
from oracle.oracle import OracleGeometry
from test_cpu_build import compare_builders
from vecgeom_gb300 import workloads as W

SQUARE_X = [-3.0, -3.0, 3.0, 3.0, -2.0, -2.0, 2.0, 2.0]
SQUARE_Y = [-3.0, 3.0, 3.0, -3.0, -2.0, 2.0, 2.0, -2.0]
INVALID = {
    "opposite orientations": (SQUARE_X[:4] + [-2.0, 2.0, 2.0, -2.0], SQUARE_Y[:4] + [-2.0, -2.0, 2.0, 2.0], 5.0),
    "crossing segments": ([-3.0, 3.0, -3.0, 3.0] + SQUARE_X[4:], [-3.0, 3.0, 3.0, -3.0] + SQUARE_Y[4:], 5.0),
    "non-convex base": ([-3.0, -3.0, -1.0, 3.0] + SQUARE_X[4:], [-3.0, 3.0, 0.0, -3.0] + SQUARE_Y[4:], 5.0),
    "zero half-length": (SQUARE_X, SQUARE_Y, 0.0),
}


def _accepts(vx, vy, dz):
    g = vg.Geometry()
    try:
        g.add_gentrap(vx, vy, dz)
        return True
    except vg.VGError:
        return False


@pytest.mark.parametrize("name", sorted(W.GENTRAPS))
def test_valid_shapes_accepted(name):
    vx, vy, dz = W.GENTRAPS[name]
    assert OracleGeometry.gentrap_valid(vx, vy, dz)
    assert _accepts(vx, vy, dz)


@pytest.mark.parametrize("name", sorted(INVALID))
def test_invalid_shapes_rejected(name):
    vx, vy, dz = INVALID[name]
    assert not OracleGeometry.gentrap_valid(vx, vy, dz)
    assert not _accepts(vx, vy, dz)


def test_acceptance_agrees_on_perturbed_vertices():
    rng = np.random.default_rng(7)
    base_x, base_y = np.array(SQUARE_X), np.array(SQUARE_Y)
    agree = accepted = 0
    for k in range(400):
        vx = base_x + rng.normal(0.0, 1.5, 8)
        vy = base_y + rng.normal(0.0, 1.5, 8)
        if k % 3 == 0:  # anticlockwise input
            vx[[1, 3]], vy[[1, 3]] = vx[[3, 1]], vy[[3, 1]]
            vx[[5, 7]], vy[[5, 7]] = vx[[7, 5]], vy[[7, 5]]
        o = OracleGeometry.gentrap_valid(vx, vy, 5.0)
        p = _accepts(vx, vy, 5.0)
        agree += o == p
        accepted += p
    assert agree == 400 and 50 < accepted < 400, (agree, accepted)


def test_anticlockwise_equals_its_clockwise_order():
    vx, vy, dz = W.GENTRAPS["anticlockwise"]
    cx, cy = list(vx), list(vy)
    for a, b in ((1, 3), (5, 7)):
        cx[a], cx[b] = cx[b], cx[a]
        cy[a], cy[b] = cy[b], cy[a]
    o = OracleGeometry()
    s1, s2 = o.add_gentrap(vx, vy, dz), o.add_gentrap(cx, cy, dz)
    rng = np.random.default_rng(3)
    n = 20000
    p = [rng.uniform(-45.0, 45.0, n), rng.uniform(-45.0, 45.0, n), rng.uniform(-40.0, 40.0, n)]
    d = rng.normal(size=(3, n))
    d /= np.linalg.norm(d, axis=0)
    for q in range(6):
        a = o.shape_query(s1, q, *p, *d)
        b = o.shape_query(s2, q, *p, *d)
        assert np.array_equal(np.asarray(a).view(np.int64) if q > 1 else a,
                              np.asarray(b).view(np.int64) if q > 1 else b), q
    assert np.array_equal(np.array(o.shape_extent(s1)), np.array(o.shape_extent(s2)))


def test_gentrap_ring_builds_identically():
    compare_builders(W.build_gentrap_ring)


# The twisted trapezoid of the reference's unit test (TestGenTrap.cpp trap2).
TRAP2 = ([-3.0, -3.0, 3.0, 3.0, -2.0, -2.0, 2.0, 2.0], [-3.0, 3.0, 3.0, -3.0, -1.9, 2.0, 2.0, -2.0], 5.0)


def surface_points(vx, vy, dz, n, seed):
    """Seeded points on the GenTrap's surface, drawn as UnplacedGenTrap::SamplePointOnSurface
    draws them (source/UnplacedGenTrap.cpp:20-124): a face chosen uniformly among the six; on
    a lateral face the bilinear point a + fz vi + f h0 + f fz (vj - vi) for uniform f, fz; on
    a base a uniform point of its bounding rectangle kept when inside the polygon. The
    vertices must be in clockwise order."""
    rng = np.random.default_rng(seed)
    v = np.array([[vx[i], vy[i], -dz if i < 4 else dz] for i in range(8)])
    out = []
    while len(out) < n:
        face = int(rng.integers(0, 6))
        if face < 4:
            j = (face + 1) % 4
            vi, vj, h0 = v[face + 4] - v[face], v[j + 4] - v[j], v[j] - v[face]
            fz, f = rng.random(), rng.random()
            out.append(v[face] + fz * vi + f * h0 + f * fz * (vj - vi))
            continue
        b = v[4 * (face - 4):4 * (face - 4) + 4]
        x, y = rng.uniform(b[:, 0].min(), b[:, 0].max()), rng.uniform(b[:, 1].min(), b[:, 1].max())
        ok = all((x - b[k, 0]) * (b[(k + 1) % 4, 1] - b[k, 1]) - (y - b[k, 1]) * (b[(k + 1) % 4, 0] - b[k, 0])
                 >= -1e-9 for k in range(4))
        if ok:
            out.append(np.array([x, y, b[0, 2]]))
    return np.array(out)


def shooting_rays(n, seed):
    """The unit test's surface-shooting check: from 100 x psurf towards psurf (expected
    distance |psurf - start|), and from psurf away (expected kInfLength)."""
    ps = surface_points(*TRAP2, n, seed)
    start = 100.0 * ps
    d = ps - start
    dist = np.linalg.norm(d, axis=1)
    d = d / dist[:, None]
    return ps, start, d, dist


def test_oracle_shoots_surface_points():
    import golden_util as G
    o = OracleGeometry()
    s = o.add_gentrap(*TRAP2)
    ps, start, d, dist = shooting_rays(2000, 11)
    into = o.shape_query(s, 2, *start.T.copy(), *d.T.copy())
    back = o.shape_query(s, 2, *ps.T.copy(), *(-d).T.copy())
    assert all(G.approx_equal(a, b) for a, b in zip(into, dist))
    assert all(G.approx_equal(a, np.finfo(np.float64).max) for a in back)
