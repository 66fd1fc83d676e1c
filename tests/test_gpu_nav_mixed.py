"""GPU parity of the mixed-precision navigator (VG_PREC_MIXED) against the FP64 oracle:
out-states bit-identical and steps within 1e-9 mm + 1e-12 rel, on the barrel and on the
config-4 detector, for single steps and multi-step transport."""
import numpy as np
import pytest

from conftest import dist_mismatch

pytestmark = pytest.mark.gpu
MIXED = 1


def _dev(torch, arrs):
    return [torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in arrs]


def _locate(torch, g, pts):
    import vecgeom_gb300 as vg
    st = torch.empty(len(pts[0]) * 12, dtype=torch.uint8, device="cuda:0")
    g.locate_point(*_dev(torch, pts), st)
    return st, st.cpu().numpy().view(vg.NAVSTATE_DTYPE)


def _step(torch, g, pts, dirs, st, flags):
    import vecgeom_gb300 as vg
    n = len(pts[0])
    out = torch.empty(n * 12, dtype=torch.uint8, device="cuda:0")
    step = torch.empty(n, dtype=torch.float64, device="cuda:0")
    status = torch.empty(n, dtype=torch.int32, device="cuda:0")
    g.compute_step_and_next_volume(*_dev(torch, (*pts, *dirs)), st, out, step, status=status, flags=flags)
    return out.cpu().numpy().view(vg.NAVSTATE_DTYPE), step.cpu().numpy(), status.cpu().numpy()


@pytest.fixture(scope="module", params=["barrel", "detector"])
def geo(request, cuda):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    g, o = vg.Geometry(), OracleGeometry()
    build = W.build_barrel if request.param == "barrel" else W.build_detector
    build(g)
    build(o)
    return request.param, g, o


def _spread(n, seed, rmax, zmax):
    from vecgeom_gb300 import workloads as W
    gg = W.rng(seed, 1)
    r = rmax * np.sqrt(gg.random(n))
    ph = 2 * np.pi * gg.random(n)
    z = zmax * (2 * gg.random(n) - 1)
    return (r * np.cos(ph), r * np.sin(ph), z), W.isotropic(W.rng(seed, 2), n)


def test_mixed_single_step_everywhere(cuda, geo):
    name, g, o = geo
    pts, dirs = _spread(1 << 16, 71, 1250.0, 2950.0 if name == "detector" else 400.0)
    st, st_h = _locate(cuda, g, pts)
    ref_st, _ = o.locate(*pts, nthreads=8)
    assert np.array_equal(st_h, ref_st)
    out, step, status = _step(cuda, g, pts, dirs, st, MIXED)
    ref_out, ref_step, _, _ = o.step(*pts, *dirs, ref_st, nthreads=8)
    assert (status == 0).all()
    bad = out != ref_out
    assert not bad.any(), (int(bad.sum()), out[bad][:3], ref_out[bad][:3])
    assert not dist_mismatch(step, ref_step).any()


def test_mixed_transport_matches_oracle(cuda, geo):
    """Straight tracks from the origin, 40 steps, mixed precision: every step's state and
    length agree with the FP64 oracle."""
    from vecgeom_gb300 import workloads as W
    name, g, o = geo
    n = 8192
    (x, y, z), dirs = W.primaries_eta_phi(n, seed=81)
    st, _ = _locate(cuda, g, (x, y, z))
    ref_st, _ = o.locate(x, y, z)
    for k in range(40):
        alive = ref_st["nav_ind"] != 0
        if not alive.any():
            break
        out, step, status = _step(cuda, g, (x, y, z), dirs, st, MIXED)
        ref_out, ref_step, _, _ = o.step(x, y, z, *dirs, ref_st, nthreads=8)
        assert (status[alive] == 0).all()
        assert np.array_equal(out[alive], ref_out[alive]), k
        assert not dist_mismatch(step[alive], ref_step[alive]).any(), k
        x = np.where(alive, x + ref_step * dirs[0], x)
        y = np.where(alive, y + ref_step * dirs[1], y)
        z = np.where(alive, z + ref_step * dirs[2], z)
        ref_st = np.where(alive, ref_out, ref_st)
        st = cuda.from_numpy(ref_st.view(np.uint8).reshape(-1).copy()).to("cuda:0")


def test_mixed_equals_fp64_on_device(cuda, geo):
    """Mixed and FP64 kernels on the same 2^18 tracks: identical states and steps."""
    name, g, o = geo
    pts, dirs = _spread(1 << 18, 91, 1250.0, 2950.0 if name == "detector" else 400.0)
    st, _ = _locate(cuda, g, pts)
    o64, s64, _ = _step(cuda, g, pts, dirs, st, 0)
    o32, s32, _ = _step(cuda, g, pts, dirs, st, MIXED)
    assert np.array_equal(o64, o32)
    assert np.array_equal(s64, s32)
