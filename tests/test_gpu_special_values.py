"""Special floating-point inputs through the SoA shape kernels, whose FP64 compares and
minima run on the integer pipe: signed zeros, points exactly on surfaces, denormals, huge
values, infinities and NaNs in the points; signed zeros and denormals in the components of
unit directions.
The FP64 kernels must return what the oracle's IEEE arithmetic returns (NaN where it
returns NaN), and the mixed kernels what the FP64 kernels return (full-phi Tube safeties:
never above it and within their stated bound). (Non-finite and zero
directions are left out: the shapes assume unit directions and take sgn(d), and the sign
of a NaN the arithmetic generates is not specified by IEEE 754 and differs between CPUs
and the GPU.)"""
import numpy as np
import pytest

from test_gpu_shapes import oracle_all, run_all_queries

pytestmark = pytest.mark.gpu

SHAPES = {
    "box": ("box", (10.0, 20.0, 30.0)),
    "tube": ("tube", (10.0, 20.0, 30.0, 0.0, 2 * np.pi)),
    "tube_phi": ("tube", (10.0, 20.0, 30.0, 0.3, 1.8)),
    "cone": ("cone", (5.0, 10.0, 8.0, 15.0, 25.0, 0.0, 2 * np.pi)),
    "trd": ("trd", (30.0, 10.0, 40.0, 15.0, 60.0)),
    "trap": ("trap", (60.0, 0.1, 0.4, 40.0, 20.0, 30.0, 0.15, 50.0, 25.0, 35.0, 0.15)),
}


def special_inputs(dims):
    vals = [0.0, -0.0, 5e-324, -5e-324, 1e-300, 1.0, -1.0, 1e300, -1e300, np.inf, -np.inf, np.nan]
    vals += [float(v) for v in dims] + [-float(v) for v in dims]
    g = np.random.default_rng(99)
    n = 4096
    pts = [g.choice(vals, n) for _ in range(3)]
    # half of the points ordinary, with one special coordinate
    ordinary = g.uniform(-40.0, 40.0, (3, n))
    for k in range(3):
        keep = g.random(n) < 0.5
        pts[k] = np.where(keep, ordinary[k], pts[k])
    # unit directions (the shapes assume them); a quarter of the components are set to +-0
    # or a denormal and the remaining ones renormalised (at least one stays ordinary)
    d = g.normal(size=(3, n))
    sel = g.random((3, n)) < 0.25
    sel[2, sel.all(axis=0)] = False
    keep = np.where(sel, 0.0, d)
    keep /= np.linalg.norm(keep, axis=0)
    d = np.where(sel, g.choice(np.array([0.0, -0.0, 5e-324, -5e-324]), (3, n)), keep)
    dirs = [d[k] for k in range(3)]
    return tuple(np.ascontiguousarray(a) for a in pts), tuple(np.ascontiguousarray(a) for a in dirs)


@pytest.mark.parametrize("name", sorted(SHAPES))
def test_special_values_fp64_and_mixed(cuda, name):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    kind, params = SHAPES[name]
    g, o = vg.Geometry(), OracleGeometry()
    s, pv = W.build_single_shape(g, kind, params)
    W.build_single_shape(o, kind, params)
    pts, dirs = special_inputs(params[:3])
    gpu = run_all_queries(cuda, g, pv, pts, dirs)
    ref = oracle_all(o, pv, pts, dirs)
    for q in (0, 1):
        assert np.array_equal(gpu[q], ref[q]), (name, q, int((gpu[q] != ref[q]).sum()))
    for q in (2, 3, 4, 5):
        a, b = gpu[q], ref[q]
        assert np.array_equal(np.isnan(a), np.isnan(b)), (name, q)
        fin = ~np.isnan(a)
        assert np.array_equal(a[fin], b[fin]), (name, q, int((a[fin] != b[fin]).sum()))
    mixed = run_all_queries(cuda, g, pv, pts, dirs, flags=vg.PREC_MIXED)
    for q in (0, 1, 2, 3):
        assert np.array_equal(mixed[q], gpu[q], equal_nan=q >= 2), (name, q)
    full_tube = kind == "tube" and params[4] >= 2 * np.pi
    for q in (4, 5):
        if not full_tube:
            assert np.array_equal(mixed[q], gpu[q], equal_nan=True), (name, q)
            continue
        # full-phi Tube: the FP32 form (points within 4 m) never exceeds the FP64 value and
        # stays within its bound below it; every other point takes the FP64 kernel
        same = (mixed[q] == gpu[q]) | (np.isnan(mixed[q]) & np.isnan(gpu[q]))
        with np.errstate(invalid="ignore", over="ignore"):
            r = np.hypot(pts[0], pts[1])
            bound = 2.0 ** -20 * (np.maximum(r, np.abs(pts[2])) + max(params[1], params[2]))
            ok = same | ((mixed[q] <= gpu[q]) & (gpu[q] - mixed[q] <= bound * 1.0001))
        assert ok.all(), (name, q, int((~ok).sum()))
        assert (~same).any(), (name, q)
