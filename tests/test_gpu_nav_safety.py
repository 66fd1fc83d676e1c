"""Step + safety (ComputeStepAndSafetyAndPropagatedState with the BVH safety estimator)
against the FP64 oracle: safeties equal, out-states bit-identical, steps within
1e-9 mm + 1e-12 relative, in FP64 and in mixed precision, on the barrel and the detector."""
import numpy as np
import pytest

from conftest import dist_mismatch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["barrel", "detector"])
def geo(request, cuda):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    g, o = vg.Geometry(), OracleGeometry()
    b = W.build_barrel if request.param == "barrel" else W.build_detector
    b(g)
    b(o)
    return request.param, g, o


@pytest.mark.parametrize("prec", [0, 1])
def test_step_and_safety_match_oracle(cuda, geo, prec):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    name, g, o = geo
    n = 1 << 15
    gg = W.rng(41, 1)
    r = 1250.0 * np.sqrt(gg.random(n))
    ph = 2 * np.pi * gg.random(n)
    zmax = 2950.0 if name == "detector" else 400.0
    pts = (r * np.cos(ph), r * np.sin(ph), zmax * (2 * gg.random(n) - 1))
    dirs = W.isotropic(W.rng(41, 2), n)
    limit = np.where(gg.random(n) < 0.3, 5.0 * gg.random(n), np.finfo(np.float64).max)
    dev = [cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (*pts, *dirs, limit)]
    st = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
    g.locate_point(*dev[:3], st)
    ref_st, _ = o.locate(*pts, nthreads=8)
    out = cuda.empty_like(st)
    step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
    saf = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
    status = cuda.empty(n, dtype=cuda.int32, device="cuda:0")
    g.compute_step_and_safety(*dev[:6], st, out, step, saf, step_limit=dev[6], status=status, flags=prec)
    ref_out, ref_step, ref_saf, _ = o.step_safety(*pts, *dirs, ref_st, step_limit=limit, nthreads=8)
    alive = ref_st["nav_ind"] != 0
    assert (status.cpu().numpy()[alive] == 0).all()
    assert np.array_equal(out.cpu().numpy().view(vg.NAVSTATE_DTYPE)[alive], ref_out[alive])
    assert not dist_mismatch(step.cpu().numpy()[alive], ref_step[alive]).any()
    assert np.array_equal(saf.cpu().numpy()[alive], ref_saf[alive])
    assert (ref_saf[alive] > 0).mean() > 0.5
