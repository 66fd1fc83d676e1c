"""Hype on the GPU, through the C-ABI, against the oracle (which passes the 84 known answers
of the reference's TestHype): the six SoA queries, FP64 and mixed, on inside, outside and
near-surface points of hollow, solid, cylindrical-inner and conical-inner hyperboloids
placed with a rotation; and navigation in the hyperboloid ring: one step from sampled
transport states and whole transport streams equal the oracle, every mixed schedule equals
plain FP64."""
import os

import numpy as np
import pytest

from conftest import dist_mismatch

pytestmark = pytest.mark.gpu
QUERIES = ["inside", "contains", "distance_to_in", "distance_to_out", "safety_to_in", "safety_to_out"]
NAMES = ["hollow", "solid", "cylinder_in", "cone_in"]


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


@pytest.mark.parametrize("name", NAMES)
def test_hype_queries_match_oracle(cuda, name):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    g, o = vg.Geometry(), OracleGeometry()
    s = g.add_hype(*W.HYPES[name])
    pv = g.place(g.add_logical_volume(s), (2.0, -1.0, 3.0), W.rot_z(0.3))
    g.close()
    so = o.add_hype(*W.HYPES[name])
    opv = o.place(o.add_logical_volume(so), (2.0, -1.0, 3.0), W.rot_z(0.3))
    o.close()
    lo, hi = g.shape_extent(s)
    lo, hi = np.asarray(lo) - 8.0, np.asarray(hi) + 8.0
    pts, dirs = W.shape_points_mixed(lo, hi, 3 * 8192, 950 + NAMES.index(name),
                                     lambda x, y, z: o.query(opv, 0, x, y, z)[0], lambda *a: o.query(opv, 3, *a)[0])
    a = _run(cuda, g, pv, pts, dirs, vg.PREC_FP64)
    b = _run(cuda, g, pv, pts, dirs, vg.PREC_MIXED)
    for qi, q in enumerate(QUERIES):
        ref = o.query(opv, qi, *pts, *(dirs if qi in (2, 3) else ()))[0]
        if qi < 2:
            assert np.array_equal(a[q].astype(np.int32), ref.astype(np.int32)), q
        else:
            bad = dist_mismatch(a[q], ref)
            assert not bad.any(), (q, int(bad.sum()), a[q][bad][:3], ref[bad][:3])
        assert np.array_equal(a[q], b[q]), (q, "mixed")
    assert {1, 3} <= set(np.unique(a["inside"]).tolist())


def test_hype_navigation_matches_oracle(cuda):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry, transport_step_sample
    from vecgeom_gb300 import workloads as W
    g, o = vg.Geometry(), OracleGeometry()
    W.build_hype_ring(g)
    W.build_hype_ring(o)
    nt = os.cpu_count() or 1
    cols, st, _ = transport_step_sample(o, 1 << 16, 0x4E9, 1 << 16, nthreads=nt)
    n = len(st)
    t = [cuda.from_numpy(np.ascontiguousarray(c)).to("cuda:0") for c in cols]
    sin = cuda.from_numpy(np.frombuffer(st.tobytes(), dtype=np.uint8).copy()).to("cuda:0")
    ref_out, ref_step, _, _ = o.step(*cols, st, nthreads=nt)
    outs = {}
    for flags in (vg.PREC_FP64, vg.PREC_MIXED, vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE):
        out = cuda.empty_like(sin)
        step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
        g.compute_step_and_next_volume(*t, sin, out, step, flags=flags)
        outs[flags] = (out.cpu().numpy().view(vg.NAVSTATE_DTYPE), step.cpu().numpy())
    got, gstep = outs[vg.PREC_FP64]
    for f in ("nav_ind", "last_exited", "on_boundary"):
        assert np.array_equal(got[f], ref_out[f]), f
    assert not dist_mismatch(gstep, ref_step).any()
    for flags, (o2, s2) in outs.items():
        assert np.array_equal(o2, got) and np.array_equal(s2, gstep), flags
    (x, y, z), (dx, dy, dz), _ = W.stream_tracks(4096, 0x4EA, world_half=(600.0, 600.0, 400.0))
    dev = [cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (x, y, z, dx, dy, dz)]
    s0 = cuda.empty(4096 * 12, dtype=cuda.uint8, device="cuda:0")
    g.locate_point(*dev[:3], s0)
    ref_st, _ = o.locate(x, y, z, nthreads=nt)
    assert np.array_equal(s0.cpu().numpy().view(vg.NAVSTATE_DTYPE)["nav_ind"], ref_st["nav_ind"])
    nsteps, status, _, _, _ = g.transport(*dev, s0, max_steps=200, flags=vg.PREC_FP64)
    ref_n, ref_final, _, _, _ = o.transport(x, y, z, dx, dy, dz, ref_st, 200, nthreads=nt)
    assert (status.cpu().numpy() == 0).all()
    assert np.array_equal(nsteps.cpu().numpy(), ref_n)
    assert np.array_equal(s0.cpu().numpy().view(vg.NAVSTATE_DTYPE)["nav_ind"], ref_final["nav_ind"])
