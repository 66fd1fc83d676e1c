"""Config-5 transport stream on the config-4 detector: the plain FP64 stream agrees step for
step with the FP64 oracle's transport loop, and the mixed-precision, sorted, work-queue
stream with learned proposals gives the same steps, states and positions as the plain FP64
stream."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def det(cuda):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    g, o = vg.Geometry(), OracleGeometry()
    W.build_detector(g)
    W.build_detector(o)
    return g, o


def _tracks(cuda, g, n, seed):
    from vecgeom_gb300 import workloads as W
    pts, dirs, restart = W.stream_tracks(n, seed)
    dev = [cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (*pts, *dirs)]
    st = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
    g.locate_point(*dev[:3], st)
    return pts, dirs, restart, dev, st


def test_fp64_stream_matches_oracle_step_for_step(cuda, det):
    import vecgeom_gb300 as vg
    g, o = det
    n, max_steps = 2048, 400
    pts, dirs, restart, dev, st = _tracks(cuda, g, n, 55)
    assert 0.1 < restart.mean() < 0.3
    ref_st, _ = o.locate(*pts, nthreads=8)
    assert np.array_equal(st.cpu().numpy().view(vg.NAVSTATE_DTYPE), ref_st)
    nsteps, status, iters, tst, tsp = g.transport(*dev, st, max_steps=max_steps, flags=vg.PREC_FP64,
                                                   trace_tracks=n)
    ref_n, ref_final, ref_tr, ref_ts, _ = o.transport(*pts, *dirs, ref_st, max_steps, trace=True, nthreads=8)
    ns = nsteps.cpu().numpy()
    assert (status.cpu().numpy() == 0).all()
    assert np.array_equal(ns, ref_n)
    assert ns.max() > 20 and iters == ns.max()
    assert np.array_equal(st.cpu().numpy().view(vg.NAVSTATE_DTYPE), ref_final)
    trs = tst.cpu().numpy().view(vg.NAVSTATE_DTYPE).reshape(n, max_steps)["nav_ind"]
    tsl = tsp.cpu().numpy().reshape(n, max_steps)
    mask = np.arange(max_steps)[None, :] < ns[:, None]
    assert np.array_equal(trs[mask], ref_tr[mask])
    assert np.array_equal(tsl[mask], ref_ts[mask])


def test_mixed_learned_stream_identical_to_fp64(cuda, det):
    """Proposals only change the order of the exact traversal, so even an untrained model
    must leave every step unchanged."""
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import learned as L
    g, o = det
    model = L.Proposer(g, seed=99)
    model.attach(g)
    n, max_steps, ntr = 1 << 16, 400, 512
    res = []
    for flags in (vg.PREC_FP64, vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE | vg.NAV_LEARNED):
        pts, dirs, restart, dev, st = _tracks(cuda, g, n, 77)
        nsteps, status, iters, tst, tsp = g.transport(*dev, st, max_steps=max_steps, flags=flags, trace_tracks=ntr)
        res.append([a.cpu().numpy() for a in (nsteps, status, st, dev[0], dev[1], dev[2], tst, tsp)])
    assert model.error() == 0
    for a, b in zip(*res):
        assert np.array_equal(a, b)
    assert res[0][0].sum() > 10 * n



def test_device_loop_stopping_rule(cuda, det):
    """The device-side loop stops where the host rule stops: after max_steps iterations (odd
    and even counts, so either half of the graph body is the last), when no track is alive,
    and, with the work queue, as soon as fewer tracks are alive than the tail pass holds.
    Truncated runs equal the oracle's transport with the same max_steps; max_steps = 0
    leaves every track where it is."""
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import learned as L
    g, o = det
    L.Proposer(g, seed=5).attach(g)
    n = 2048
    pts, dirs, restart, dev, st0 = _tracks(cuda, g, n, 91)
    ref_st, _ = o.locate(*pts, nthreads=8)
    loops = (vg.PREC_FP64, vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_LEARNED)
    for max_steps in (0, 1, 2, 3, 7):
        ref_n, ref_final, _, _, _ = o.transport(*pts, *dirs, ref_st, max_steps, trace=False, nthreads=8)
        for flags in loops + (vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE,):
            d = [a.clone() for a in dev]
            st = st0.clone()
            nsteps, status, iters, _, _ = g.transport(*d, st, max_steps=max_steps, flags=flags)
            ns = nsteps.cpu().numpy()
            assert np.array_equal(ns, ref_n), (max_steps, flags)
            assert np.array_equal(st.cpu().numpy().view(vg.NAVSTATE_DTYPE), ref_final), (max_steps, flags)
            # 2048 live tracks are fewer than the tail pass holds: with the queue it takes
            # them at once; otherwise one iteration per step of the longest track
            assert iters == (min(max_steps, 1) if flags & vg.NAV_QUEUE else ns.max()), (max_steps, flags, iters)
            moved = not np.array_equal(d[0].cpu().numpy(), pts[0])
            assert moved == (max_steps > 0)
    for flags in loops:  # untruncated: the loop ends when no track is alive
        d = [a.clone() for a in dev]
        st = st0.clone()
        nsteps, _, iters, _, _ = g.transport(*d, st, max_steps=400, flags=flags)
        assert iters == nsteps.cpu().numpy().max() > 20


def test_device_loop_then_tail_pass(cuda, det):
    """With the work queue and more live tracks than the tail pass holds (152 x 512), the loop
    iterates on the device until the survivors fit, then the tail pass finishes them: same
    results as the plain FP64 stream."""
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import learned as L
    g, o = det
    L.Proposer(g, seed=6).attach(g)
    n = 1 << 17
    res = []
    for flags in (vg.PREC_FP64, vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE | vg.NAV_LEARNED):
        pts, dirs, restart, dev, st = _tracks(cuda, g, n, 93)
        nsteps, status, iters, _, _ = g.transport(*dev, st, max_steps=400, flags=flags)
        res.append(([a.cpu().numpy() for a in (nsteps, status, st, dev[0], dev[1], dev[2])], iters))
    (a, it64), (b, itq) = res
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    assert it64 == a[0].max()
    assert 1 < itq < it64
