"""The unplaced (shape-frame) SoA queries, vg_shape_*: points and directions go to the shape
kernels untransformed (VUnplacedVolume), so signed zeros reach the kernels as given. Against
the oracle's unplaced queries: bit-exact in FP64 (Torus2 distances within 1e-9 mm + 1e-12
relative), and the
mixed-precision results equal to FP64 (full-phi Tube safeties excepted: their FP32 form has a stated
bound)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = ["box", "tube_phi", "cone", "trd", "trap", "polycone", "polyhedron", "torus2", "box_minus_tube"]
QUERIES = ["inside", "contains", "distance_to_in", "distance_to_out", "safety_to_in", "safety_to_out"]


def _spec(name):
    from vecgeom_gb300 import workloads as W
    if name in W.SHAPES_CFG1:
        return W.SHAPES_CFG1[name]
    if name == "trap":
        return ("trap", W.TRAP_WEDGE)
    return W.SHAPES_CFG2[name]


def _points(lo, hi, n, seed):
    from vecgeom_gb300 import workloads as W
    (x, y, z), (dx, dy, dz) = W.shape_points_box(lo, hi, n, seed)
    g = np.random.default_rng(seed)
    pts = [np.where(g.random(n) < 0.1, -0.0, a) for a in (x, y, z)]
    d = np.stack([dx, dy, dz])
    zero = g.random((3, n)) < 0.1
    zero[2, zero.all(axis=0)] = False
    d = np.where(zero, 0.0, d)
    d /= np.linalg.norm(d, axis=0)
    d = np.where(zero, np.where(g.random((3, n)) < 0.5, -0.0, 0.0), d)
    return [np.ascontiguousarray(a) for a in pts], [np.ascontiguousarray(a) for a in d]


@pytest.mark.parametrize("name", SHAPES)
def test_unplaced_queries_match_oracle(cuda, name):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    kind, params = _spec(name)
    g, o = vg.Geometry(), OracleGeometry()
    s, _ = W.build_single_shape(g, kind, params)
    so, _ = W.build_single_shape(o, kind, params)
    assert s == so
    lo, hi = g.shape_extent(s)
    pts, dirs = _points(lo, hi, 1 << 15, 81)
    dev = lambda a: cuda.from_numpy(a).to("cuda:0")
    t = [dev(a) for a in (*pts, *dirs)]
    n = len(pts[0])
    res = {}
    for flags in (vg.PREC_FP64, vg.PREC_MIXED):
        for qi, q in enumerate(QUERIES):
            dt = {0: cuda.int32, 1: cuda.uint8}.get(qi, cuda.float64)
            out = cuda.empty(n, dtype=dt, device="cuda:0")
            if qi in (2, 3):
                g.shape_query(q, s, *t[:3], out, *t[3:], flags=flags)
            else:
                g.shape_query(q, s, *t[:3], out, flags=flags)
            res[flags, qi] = out.cpu().numpy().astype(np.int32 if qi < 2 else np.float64)
    for qi in range(6):
        ref = o.shape_query(so, qi, *pts, *(dirs if qi in (2, 3) else ()))
        got = res[vg.PREC_FP64, qi]
        if kind == "torus2" and qi in (2, 3):
            bad = ~((got == ref) | (np.abs(got - ref) <= 1e-9 + 1e-12 * np.abs(ref)))
        else:
            bad = ~((got == ref) | (np.isnan(got) & np.isnan(ref)))
        assert not bad.any(), (name, QUERIES[qi], int(bad.sum()), got[bad][:3], ref[bad][:3])
        if not (kind == "tube" and params[4] >= 2 * np.pi and qi >= 4):
            assert np.array_equal(res[vg.PREC_MIXED, qi], got, equal_nan=True), (name, QUERIES[qi])
