"""BVH::ApproachNextDaughter on the GPU (vg_nav_approach_next_daughter) against the oracle,
bit-exact, on the config-3 barrel and on the GDML detector: from located track starts with an
unbounded and a finite step, and from the boundary states a step leaves (so the last-exited
volume is excluded). Property: when the step enters a daughter, the approach distance to
that daughter's bounding box is no longer than the step."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DETECTOR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gdml", "detector.gdml")


def _geoms(name):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import gdml
    from vecgeom_gb300 import workloads as W
    g, o = vg.Geometry(), OracleGeometry()
    if name == "barrel":
        W.build_barrel(g)
        W.build_barrel(o)
        rmax, halfz = 1250.0, 400.0
    else:
        gdml.load(DETECTOR, g)
        gdml.load(DETECTOR, o)
        rmax, halfz = 1400.0, 1900.0
    return g, o, rmax, halfz


@pytest.mark.parametrize("name", ["barrel", "gdml"])
def test_approach_next_daughter_matches_oracle(cuda, name):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    g, o, rmax, halfz = _geoms(name)
    n = 1 << 15
    gg = np.random.default_rng(71)
    r = rmax * np.sqrt(gg.random(n))
    ph = 2 * np.pi * gg.random(n)
    pts = [r * np.cos(ph), r * np.sin(ph), halfz * (2 * gg.random(n) - 1)]
    dirs = list(W.isotropic(W.rng(71, 1), n))
    dev = lambda a: cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0")
    st_h, _ = o.locate(*pts, nthreads=8)
    out_h, step_h, _, _ = o.step(*pts, *dirs, st_h, nthreads=8)
    cases = [(pts, st_h, np.full(n, np.finfo(np.float64).max)), (pts, st_h, gg.uniform(0.0, 80.0, n))]
    # from the boundary a step reaches: moved points, out-states with last-exited set
    moved = [pts[k] + step_h * dirs[k] for k in range(3)]
    cases.append((moved, out_h, np.full(n, np.finfo(np.float64).max)))
    for k, (p, st, s0) in enumerate(cases):
        ref = o.approach_next_daughter(*p, *dirs, st, s0, nthreads=8)
        step = dev(s0)
        status = cuda.empty(n, dtype=cuda.int32, device="cuda:0")
        sd = dev(st.view(np.uint8).reshape(-1))
        g.approach_next_daughter(*(dev(a) for a in (*p, *dirs)), sd, step, status)
        got, stat = step.cpu().numpy(), status.cpu().numpy()
        alive = st["nav_ind"] != 0
        assert (stat[alive] == 0).all() and (stat[~alive] == 3).all(), k
        assert np.array_equal(got, ref), (k, int((got != ref).sum()))
        assert (ref[alive] < s0[alive]).mean() > 0.03, k
    # entering a daughter: the box of that daughter is reached no later than the daughter
    ref = o.approach_next_daughter(*pts, *dirs, st_h, np.full(n, np.finfo(np.float64).max), nthreads=8)
    # the step entered a daughter when the start state is a proper ancestor of the out-state
    # (NavIndex table: word n holds the parent of node n)
    table = o.nav_table()
    a = out_h["nav_ind"].astype(np.int64)
    entering = np.zeros(n, bool)
    for _ in range(8):
        a = np.where(a != 0, table[a], 0)
        entering |= (a == st_h["nav_ind"]) & (st_h["nav_ind"] != 0)
    assert entering.sum() > 100
    assert (ref[entering] <= step_h[entering] + 1e-9).all()
