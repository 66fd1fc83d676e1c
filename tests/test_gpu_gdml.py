"""Navigation in a geometry read from GDML (tests/golden/gdml/detector.gdml: boxes in a
barrel tube, Trd wedges in polycone endcaps, trapezoids in a polyhedra, a torus, a phi-cut
cone and a boolean subtraction, with rotations from GDML angles): LocatePoint and the
transport stream step for step equal to the oracle (FP64: states bit-exact, steps bit-exact
except at the Torus2, within 1e-9 mm + 1e-12 relative there), and every mixed-precision schedule equal to
FP64."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DETECTOR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gdml", "detector.gdml")


@pytest.fixture(scope="module")
def gdml_det(cuda):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import gdml
    g, o = vg.Geometry(), OracleGeometry()
    gdml.load(DETECTOR, g)
    gdml.load(DETECTOR, o)
    return g, o


def _tracks(cuda, n, seed):
    from vecgeom_gb300 import workloads as W
    gg = np.random.default_rng(seed)
    # half of the starts in the barrel and endcap region, half anywhere in the world
    inner = gg.random(n) < 0.5
    r = np.where(inner, 600.0, 1450.0) * np.sqrt(gg.random(n))
    ph = 2 * np.pi * gg.random(n)
    pts = (r * np.cos(ph), r * np.sin(ph), np.where(inner, 1100.0, 1950.0) * (2 * gg.random(n) - 1))
    dirs = W.isotropic(W.rng(seed, 3), n)
    dev = [cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (*pts, *dirs)]
    return pts, dirs, dev


def test_gdml_locate_and_transport_match_oracle(cuda, gdml_det):
    import vecgeom_gb300 as vg
    g, o = gdml_det
    n, max_steps = 4096, 200
    pts, dirs, dev = _tracks(cuda, n, 61)
    st = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
    g.locate_point(*dev[:3], st)
    ref_st, _ = o.locate(*pts, nthreads=8)
    assert np.array_equal(st.cpu().numpy().view(vg.NAVSTATE_DTYPE), ref_st)
    nsteps, status, iters, tst, tsp = g.transport(*dev, st, max_steps=max_steps, flags=vg.PREC_FP64, trace_tracks=n)
    ref_n, ref_final, ref_tr, ref_ts, _ = o.transport(*pts, *dirs, ref_st, max_steps, trace=True, nthreads=8)
    ns = nsteps.cpu().numpy()
    assert (status.cpu().numpy() == 0).all()
    assert np.array_equal(ns, ref_n)
    assert np.array_equal(st.cpu().numpy().view(vg.NAVSTATE_DTYPE), ref_final)
    trs = tst.cpu().numpy().view(vg.NAVSTATE_DTYPE).reshape(n, max_steps)["nav_ind"]
    tsl = tsp.cpu().numpy().reshape(n, max_steps)
    mask = np.arange(max_steps)[None, :] < ns[:, None]
    assert np.array_equal(trs[mask], ref_tr[mask])
    # steps bit-exact, except the steps into or out of the Torus2 ring: its cubic solve calls
    # cbrt/pow/cos/atan2, whose CUDA and libm results differ in the last bits, so those
    # steps are compared at 1e-9 mm + 1e-12 relative (the bar of every shape)
    torus_ind = o.locate(np.array([1000.0]), np.array([0.0]), np.array([1500.0]))[0]["nav_ind"][0]
    prev = np.concatenate([ref_st["nav_ind"][:, None], ref_tr[:, :-1]], axis=1)
    differ = mask & (tsl != ref_ts)
    assert (np.abs(tsl - ref_ts)[differ] <= 1e-9 + 1e-12 * np.abs(ref_ts[differ])).all()
    assert ((ref_tr == torus_ind) | (prev == torus_ind))[differ].all()
    assert differ.sum() < 0.01 * mask.sum()
    # tracks cross the modules, wedges, trapezoids and the other daughters
    assert len(np.unique(ref_tr[mask])) > 120 and ns.sum() > 2 * n


def test_gdml_mixed_schedules_identical_to_fp64(cuda, gdml_det):
    import vecgeom_gb300 as vg
    g, _ = gdml_det
    n, max_steps, ntr = 1 << 15, 200, 256
    res = []
    for flags in (vg.PREC_FP64, vg.PREC_MIXED, vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE):
        pts, dirs, dev = _tracks(cuda, n, 62)
        st = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
        g.locate_point(*dev[:3], st)
        nsteps, status, iters, tst, tsp = g.transport(*dev, st, max_steps=max_steps, flags=flags, trace_tracks=ntr)
        res.append([a.cpu().numpy() for a in (nsteps, status, st, dev[0], dev[1], dev[2], tst, tsp)])
    for other in res[1:]:
        for a, b in zip(res[0], other):
            assert np.array_equal(a, b)
