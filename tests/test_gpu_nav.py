"""GPU parity of the FP64 BVH navigator against the oracle on the config-3 barrel:
LocatePoint states, ComputeStepAndNextVolume out-states (bit-exact, including
last-exited and on-boundary) and steps (1e-9 mm + 1e-12 rel), and multi-step transport."""
import numpy as np
import pytest

from conftest import dist_mismatch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def barrel(cuda):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W

    g, o = vg.Geometry(), OracleGeometry()
    W.build_barrel(g)
    W.build_barrel(o)
    return g, o


def to_dev(torch, arrs):
    return [torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in arrs]


def gpu_locate(torch, g, pts):
    import vecgeom_gb300 as vg
    t = to_dev(torch, pts)
    st = torch.empty(len(pts[0]) * 12, dtype=torch.uint8, device="cuda:0")
    g.locate_point(*t, st)
    return st, st.cpu().numpy().view(vg.NAVSTATE_DTYPE)


def gpu_step(torch, g, pts, dirs, st, flags=0):
    import vecgeom_gb300 as vg
    t = to_dev(torch, (*pts, *dirs))
    n = len(pts[0])
    out = torch.empty(n * 12, dtype=torch.uint8, device="cuda:0")
    step = torch.empty(n, dtype=torch.float64, device="cuda:0")
    status = torch.empty(n, dtype=torch.int32, device="cuda:0")
    g.compute_step_and_next_volume(*t, st, out, step, status=status, flags=flags)
    return out.cpu().numpy().view(vg.NAVSTATE_DTYPE), step.cpu().numpy(), status.cpu().numpy()


def random_world_tracks(n, seed):
    from vecgeom_gb300 import workloads as W
    g = W.rng(seed, 9)
    r = 1250.0 * np.sqrt(g.random(n))
    ph = 2 * np.pi * g.random(n)
    z = 400.0 * (2 * g.random(n) - 1)
    return (r * np.cos(ph), r * np.sin(ph), z), W.isotropic(W.rng(seed, 10), n)


def test_locate_and_step_cfg3_tracks(cuda, barrel):
    from vecgeom_gb300 import workloads as W
    g, o = barrel
    pts, dirs = W.tracks_in_cylinder(1 << 15, seed=21)
    st, st_h = gpu_locate(cuda, g, pts)
    ref_st, _ = o.locate(*pts)
    assert np.array_equal(st_h, ref_st)
    out, step, status = gpu_step(cuda, g, pts, dirs, st)
    ref_out, ref_step, _, _ = o.step(*pts, *dirs, ref_st)
    assert (status == 0).all()
    assert np.array_equal(out, ref_out)
    assert not dist_mismatch(step, ref_step).any()


def test_locate_and_step_everywhere(cuda, barrel):
    """Track starts spread over the whole barrel, so steps start inside layers, modules
    and sensors and cross many BVH leaves."""
    g, o = barrel
    pts, dirs = random_world_tracks(1 << 16, seed=31)
    st, st_h = gpu_locate(cuda, g, pts)
    ref_st, _ = o.locate(*pts)
    assert np.array_equal(st_h, ref_st)
    out, step, status = gpu_step(cuda, g, pts, dirs, st)
    ref_out, ref_step, _, _ = o.step(*pts, *dirs, ref_st)
    assert (status == 0).all()
    assert np.array_equal(out, ref_out)
    assert not dist_mismatch(step, ref_step).any()


def test_transport_sequence_matches(cuda, barrel):
    """Step-for-step transport: every step's out-state and step agree with the oracle."""
    from vecgeom_gb300 import workloads as W
    g, o = barrel
    n = 4096
    (x, y, z), dirs = W.tracks_in_cylinder(n, seed=41)
    st, st_h = gpu_locate(cuda, g, (x, y, z))
    ref_st, _ = o.locate(x, y, z)
    for k in range(12):
        alive = st_h["nav_ind"] != 0
        out, step, status = gpu_step(cuda, g, (x, y, z), dirs, st)
        ref_out, ref_step, _, _ = o.step(x, y, z, *dirs, ref_st)
        assert np.array_equal(out[alive], ref_out[alive]), k
        assert not dist_mismatch(step[alive], ref_step[alive]).any(), k
        # continue both from the oracle's numbers so the comparison stays per step
        x = np.where(alive, x + ref_step * dirs[0], x)
        y = np.where(alive, y + ref_step * dirs[1], y)
        z = np.where(alive, z + ref_step * dirs[2], z)
        ref_st = np.where(alive, ref_out, ref_st)
        st_h = ref_st.copy()
        st = cuda.from_numpy(st_h.view(np.uint8).reshape(-1).copy()).to("cuda:0")


@pytest.fixture(scope="module")
def detector(cuda):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W

    g, o = vg.Geometry(), OracleGeometry()
    W.build_detector(g)
    W.build_detector(o)
    return g, o


def test_detector_locate_step_transport(cuda, detector):
    """Config-4 detector (150k box modules, Polycone holders with Trd wedges): straight
    tracks from the origin are transported step by step; every step's state and length
    agree with the oracle."""
    from vecgeom_gb300 import workloads as W
    g, o = detector
    n = 8192
    (x, y, z), dirs = W.primaries_eta_phi(n, seed=51)
    st, st_h = gpu_locate(cuda, g, (x, y, z))
    ref_st, _ = o.locate(x, y, z)
    assert np.array_equal(st_h, ref_st)
    for k in range(40):
        alive = ref_st["nav_ind"] != 0
        if not alive.any():
            break
        out, step, status = gpu_step(cuda, g, (x, y, z), dirs, st)
        ref_out, ref_step, _, _ = o.step(x, y, z, *dirs, ref_st, nthreads=8)
        assert (status[alive] == 0).all()
        assert np.array_equal(out[alive], ref_out[alive]), k
        assert not dist_mismatch(step[alive], ref_step[alive]).any(), k
        x = np.where(alive, x + ref_step * dirs[0], x)
        y = np.where(alive, y + ref_step * dirs[1], y)
        z = np.where(alive, z + ref_step * dirs[2], z)
        ref_st = np.where(alive, ref_out, ref_st)
        st = cuda.from_numpy(ref_st.view(np.uint8).reshape(-1).copy()).to("cuda:0")


def test_detector_random_points(cuda, detector):
    """Track starts spread over the detector volume (barrel and endcaps)."""
    from vecgeom_gb300 import workloads as W
    g, o = detector
    n = 1 << 16
    gg = W.rng(61, 1)
    r = 1150.0 * np.sqrt(gg.random(n))
    ph = 2 * np.pi * gg.random(n)
    z = 2950.0 * (2 * gg.random(n) - 1)
    pts = (r * np.cos(ph), r * np.sin(ph), z)
    dirs = W.isotropic(W.rng(61, 2), n)
    st, st_h = gpu_locate(cuda, g, pts)
    ref_st, _ = o.locate(*pts, nthreads=8)
    assert np.array_equal(st_h, ref_st)
    out, step, status = gpu_step(cuda, g, pts, dirs, st)
    ref_out, ref_step, _, _ = o.step(*pts, *dirs, ref_st, nthreads=8)
    assert (status == 0).all()
    assert np.array_equal(out, ref_out)
    assert not dist_mismatch(step, ref_step).any()
