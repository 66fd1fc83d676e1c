"""Track ordering (VG_NAV_SORT) and the persistent work queue (VG_NAV_QUEUE): the sort key
and stable order match a numpy restatement bit for bit, and every scheduling variant gives
out-states and steps identical to the plain launch, in FP64 and in mixed precision."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spread(n, seed, rmax, zmax):
    from vecgeom_gb300 import workloads as W
    gg = W.rng(seed, 1)
    r = rmax * np.sqrt(gg.random(n))
    ph = 2 * np.pi * gg.random(n)
    z = zmax * (2 * gg.random(n) - 1)
    return (r * np.cos(ph), r * np.sin(ph), z), W.isotropic(W.rng(seed, 2), n)


@pytest.fixture(scope="module", params=["barrel", "detector"])
def geo(request, cuda):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    g = vg.Geometry()
    (W.build_barrel if request.param == "barrel" else W.build_detector)(g)
    zmax = 2950.0 if request.param == "detector" else 400.0
    # n not a multiple of the 4096-entry sort tile, to cover ragged tiles
    pts, dirs = _spread((1 << 17) + 1234, 313, 1250.0, zmax)
    dev = [cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (*pts, *dirs)]
    st = cuda.empty(len(pts[0]) * 12, dtype=cuda.uint8, device="cuda:0")
    g.locate_point(*dev[:3], st)
    return request.param, g, pts, dev, st


def _keys_numpy(g, pts, states):
    """Restatement of the sort key documented for vg_nav_sort_tracks."""
    lo, sc, cb, lb = g.sort_key_params()
    nav = g.nav_table()
    pv_lv = np.asarray(g.pv_lv, dtype=np.uint32)
    ni = states["nav_ind"].astype(np.int64)
    key = np.full(len(ni), 0xFFFFFFFF, dtype=np.uint32)
    ok = ni != 0
    lv = pv_lv[nav[ni[ok] + 1]]
    maxc = (1 << cb) - 1

    def cell(c, k):
        f = (c.astype(np.float32) - np.float32(lo[k])) * np.float32(sc[k])
        q = np.where(f > 0, np.minimum(f, np.float32(maxc)), 0).astype(np.uint32)
        return q

    def spread(v):
        out = np.zeros_like(v)
        for b in range(cb):
            out |= ((v >> b) & 1) << (3 * b)
        return out

    m = spread(cell(pts[0][ok], 0)) | (spread(cell(pts[1][ok], 1)) << 1) | (spread(cell(pts[2][ok], 2)) << 2)
    key[ok] = (lv.astype(np.uint32) << np.uint32(3 * cb)) | m
    return key


def test_sort_order_is_stable_and_keys_match(cuda, geo):
    import vecgeom_gb300 as vg
    name, g, pts, dev, st = geo
    n = dev[0].numel()
    order = cuda.empty(n, dtype=cuda.int32, device="cuda:0")
    keys = cuda.empty(n, dtype=cuda.int32, device="cuda:0")
    g.sort_tracks(*dev[:3], st, order, keys)
    o = order.cpu().numpy().view(np.uint32)
    k = keys.cpu().numpy().view(np.uint32)
    states = st.cpu().numpy().view(vg.NAVSTATE_DTYPE)
    ref = _keys_numpy(g, pts, states)
    assert np.array_equal(np.sort(o), np.arange(n, dtype=np.uint32))
    assert np.array_equal(k, ref[o])
    assert np.array_equal(o, np.argsort(ref, kind="stable").astype(np.uint32))


@pytest.mark.parametrize("prec", [0, 1])
def test_scheduling_variants_identical(cuda, geo, prec):
    import vecgeom_gb300 as vg
    name, g, pts, dev, st = geo
    n = dev[0].numel()

    def run(flags):
        out = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
        step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
        status = cuda.empty(n, dtype=cuda.int32, device="cuda:0")
        g.compute_step_and_next_volume(*dev, st, out, step, status=status, flags=flags)
        return out.cpu().numpy(), step.cpu().numpy(), status.cpu().numpy()

    base = run(prec)
    variants = [prec | vg.NAV_SORT]
    if prec == vg.PREC_MIXED:
        variants += [prec | vg.NAV_QUEUE, prec | vg.NAV_SORT | vg.NAV_QUEUE]
    for f in variants:
        got = run(f)
        for a, b in zip(base, got):
            assert np.array_equal(a, b), f


def test_tuning_configurations_identical(cuda, geo):
    """Every work-queue configuration (256 x 1, 256 x 2, 128 x 3, 128 x 5 threads x blocks per
    SM, fused or with the step split into a step and a relocation kernel) and sort-key
    resolution gives the plain FP64 results, in the step and in the transport stream;
    out-of-range settings are rejected."""
    import vecgeom_gb300 as vg
    name, g, pts, dev, st = geo
    n = dev[0].numel()

    def run(flags):
        out = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
        step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
        g.compute_step_and_next_volume(*dev, st, out, step, flags=flags)
        return out.cpu().numpy(), step.cpu().numpy()

    base = run(vg.PREC_FP64)
    m = 4096
    sub = [d[:m].clone() for d in dev]
    sst = st[: m * 12].clone()
    ref_t = g.transport(*[d.clone() for d in sub], sst.clone(), max_steps=50, flags=vg.PREC_FP64)
    try:
        for qb in range(1, 9):
            for bits in (0, 5):
                g.set_tuning(bits, qb)
                got = run(vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE)
                assert np.array_equal(got[0], base[0]) and np.array_equal(got[1], base[1]), (qb, bits)
            tst = sst.clone()
            got_t = g.transport(*[d.clone() for d in sub], tst, max_steps=50,
                                flags=vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE)
            assert cuda.equal(got_t[0], ref_t[0]), qb
        with pytest.raises(vg.VGError):
            g.set_tuning(0, 9)
        with pytest.raises(vg.VGError):
            g.set_tuning(11, 1)
    finally:
        g.set_tuning(0, 0)


def test_host_entry_sorted_queue(cuda, geo):
    import vecgeom_gb300 as vg
    name, g, pts, dev, st = geo
    n = dev[0].numel()
    h = [d.cpu().numpy() for d in dev]
    sh = st.cpu().numpy()
    out_d = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
    step_d = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
    g.compute_step_and_next_volume(*dev, st, out_d, step_d, flags=vg.PREC_MIXED)
    out_h = np.empty(n * 12, dtype=np.uint8)
    step_h = np.empty(n, dtype=np.float64)
    status_h = np.empty(n, dtype=np.int32)
    g.compute_step_and_next_volume_host(*h, sh, out_h, step_h, status=status_h,
                                        flags=vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE)
    assert np.array_equal(out_h, out_d.cpu().numpy())
    assert np.array_equal(step_h, step_d.cpu().numpy())


def test_scheduling_flag_errors(cuda, geo):
    import vecgeom_gb300 as vg
    name, g, pts, dev, st = geo
    n = dev[0].numel()
    out = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
    step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
    with pytest.raises(vg.VGError):  # the work queue exists for the mixed kernel only
        g.compute_step_and_next_volume(*dev, st, out, step, flags=vg.NAV_QUEUE)
    with pytest.raises(vg.VGError):  # unknown flag bits
        g.compute_step_and_next_volume(*dev, st, out, step, flags=vg.PREC_MIXED | 64)
    small = cuda.empty(256, dtype=cuda.uint8, device="cuda:0")
    with pytest.raises(vg.VGError):  # workspace too small
        g.compute_step_and_next_volume(*dev, st, out, step, flags=vg.NAV_SORT, workspace=small)


@pytest.mark.parametrize("flags_name", ["fp64", "mixed_sort_queue", "mixed_sort_queue_learned"])
def test_host_entry_pipelined_chunks(cuda, flags_name):
    """From 2^18 tracks with a sorted schedule the host-array entry point copies its inputs
    in four chunks and computes each chunk's sort keys and proposals as it arrives; every
    out-state, step and status equals the device entry point's (a ragged size, so the chunks
    differ in length), and so does the unsorted plain FP64 path."""
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import learned as L
    from vecgeom_gb300 import workloads as W
    flags = {"fp64": vg.PREC_FP64, "mixed_sort_queue": vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE,
             "mixed_sort_queue_learned": vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE | vg.NAV_LEARNED}[flags_name]
    g = vg.Geometry()
    W.build_barrel(g)
    model = L.Proposer(g, seed=3)  # untrained: the learned order never changes results
    model.attach(g)
    n = 3 * (1 << 17) + 777
    pts, dirs = W.tracks_in_cylinder(n, seed=99)
    dev = [cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (*pts, *dirs)]
    st = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
    g.locate_point(*dev[:3], st)
    out_d = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
    step_d = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
    status_d = cuda.empty(n, dtype=cuda.int32, device="cuda:0")
    g.compute_step_and_next_volume(*dev, st, out_d, step_d, status=status_d, flags=flags)
    h = [np.ascontiguousarray(a) for a in (*pts, *dirs)]
    out_h = np.empty(n * 12, dtype=np.uint8)
    step_h = np.empty(n, dtype=np.float64)
    status_h = np.full(n, -7, dtype=np.int32)
    for _ in range(2):  # the second call reuses the handle's staging and streams
        g.compute_step_and_next_volume_host(*h, st.cpu().numpy(), out_h, step_h, status=status_h, flags=flags)
        assert np.array_equal(out_h, out_d.cpu().numpy())
        assert np.array_equal(step_h.view(np.int64), step_d.cpu().numpy().view(np.int64))
        assert np.array_equal(status_h, status_d.cpu().numpy())
