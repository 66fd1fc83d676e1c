"""The no-allocation step entry point (fixed device scratch inside the library) against the
workspace entry point, for every valid combination of scheduling flags: two calls in a row
give the same out-states and steps (states bit-identical, steps within 1e-9 mm + 1e-12
relative), at the full capacity of 2^20 tracks as well as at a ragged size; more tracks
than the scratch holds are rejected. Collected last so that it runs after the other GPU
tests as well as alone."""
import numpy as np
import pytest

from conftest import dist_mismatch

pytestmark = pytest.mark.gpu
MAX_TRACKS = 1 << 20


@pytest.fixture(scope="module")
def barrel(cuda):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import learned as L
    from vecgeom_gb300 import workloads as W
    g = vg.Geometry()
    W.build_barrel(g)
    # an untrained proposer: the learned order never changes results, so any weights do
    model = L.Proposer(g, seed=1)
    model.attach(g)
    pts, dirs = W.tracks_in_cylinder(MAX_TRACKS, seed=2024)
    dev = [cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (*pts, *dirs)]
    st = cuda.empty(MAX_TRACKS * 12, dtype=cuda.uint8, device="cuda:0")
    g.locate_point(*dev[:3], st)
    return g, model, dev, st


def _flag_sets():
    import vecgeom_gb300 as vg
    return {
        "fp64_sort": vg.PREC_FP64 | vg.NAV_SORT,
        "mixed_queue": vg.PREC_MIXED | vg.NAV_QUEUE,
        "mixed_sort_queue": vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE,
        "mixed_learned": vg.PREC_MIXED | vg.NAV_LEARNED,
        "mixed_sort_queue_learned": vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE | vg.NAV_LEARNED,
    }


@pytest.mark.parametrize("n", [200_003, MAX_TRACKS])
@pytest.mark.parametrize("name", ["fp64_sort", "mixed_queue", "mixed_sort_queue", "mixed_learned",
                                  "mixed_sort_queue_learned"])
def test_noalloc_matches_workspace_entry(cuda, barrel, name, n):
    g, _, dev, st_all = barrel
    flags = _flag_sets()[name]
    t = [a[:n] for a in dev]
    st = st_all[: n * 12]
    ref_out = cuda.empty_like(st)
    ref_step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
    g.compute_step_and_next_volume(*t, st, ref_out, ref_step, flags=flags)
    ref_o, ref_s = ref_out.cpu().numpy(), ref_step.cpu().numpy()
    for _ in range(2):
        out = cuda.empty_like(st)
        step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
        status = cuda.empty(n, dtype=cuda.int32, device="cuda:0")
        g.compute_step_and_next_volume_noalloc(*t, st, out, step, status=status, flags=flags)
        assert (status.cpu().numpy() == 0).all()
        assert np.array_equal(out.cpu().numpy(), ref_o)
        assert not dist_mismatch(step.cpu().numpy(), ref_s).any()


def test_noalloc_rejects_more_than_capacity(cuda, barrel):
    import vecgeom_gb300 as vg
    g = barrel[0]
    n = MAX_TRACKS + 1
    t = [cuda.zeros(n, dtype=cuda.float64, device="cuda:0") for _ in range(6)]
    t[3] += 1.0
    st = cuda.zeros(n * 12, dtype=cuda.uint8, device="cuda:0")
    out = cuda.empty_like(st)
    step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
    with pytest.raises(vg.VGError, match="capacity"):
        g.compute_step_and_next_volume_noalloc(*t, st, out, step)
