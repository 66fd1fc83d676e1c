"""Coordinates beyond the FP32 pruning range: in a 20 m world whose daughters sit up to 9 m
from the origin (translations beyond 4 m are marked FP64-only, points beyond 4 m take the
FP64 traversal), every mixed-precision schedule gives the plain FP64 states and steps."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def far_world(cuda):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    g = vg.Geometry()
    world_lv = g.add_logical_volume(g.add_box(10000.0, 10000.0, 10000.0))
    box_lv = g.add_logical_volume(g.add_box(150.0, 40.0, 300.0))
    inner_lv = g.add_logical_volume(g.add_box(100.0, 20.0, 200.0))
    g.place_daughter(box_lv, inner_lv, (10.0, 0.0, 0.0))
    gg = W.rng(2024, 7)
    k = 0
    for r in (1500.0, 3500.0, 5500.0, 8500.0):
        n = int(2 * math.pi * r / 400.0)
        for j in range(n):
            phi = 2 * math.pi * j / n
            c, s = math.cos(phi), math.sin(phi)
            z = float(gg.uniform(-900.0, 900.0))
            g.place_daughter(world_lv, box_lv, (r * c, r * s, z), W.rot_z(phi))
            k += 1
    world = g.place(world_lv)
    g.set_world(world)
    g.close()
    n = 1 << 15
    pts = [gg.uniform(-9500.0, 9500.0, n) for _ in range(2)] + [gg.uniform(-1200.0, 1200.0, n)]
    dirs = W.isotropic(W.rng(2024, 8), n)
    dev = [cuda.from_numpy(np.ascontiguousarray(a)).to("cuda:0") for a in (*pts, *dirs)]
    st = cuda.empty(n * 12, dtype=cuda.uint8, device="cuda:0")
    g.locate_point(*dev[:3], st)
    return g, dev, st, k


def test_far_coordinates_mixed_equals_fp64(cuda, far_world):
    import vecgeom_gb300 as vg
    g, dev, st, k = far_world
    assert k > 100
    n = dev[0].numel()
    res = []
    for flags in (vg.PREC_FP64, vg.PREC_MIXED, vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE):
        out = cuda.empty_like(st)
        step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
        status = cuda.empty(n, dtype=cuda.int32, device="cuda:0")
        g.compute_step_and_next_volume(*dev, st, out, step, status=status, flags=flags)
        res.append((out.cpu().numpy(), step.cpu().numpy(), status.cpu().numpy()))
    for o, s, e in res[1:]:
        assert (e == 0).all()
        assert np.array_equal(o, res[0][0])
        assert np.array_equal(s, res[0][1])
    # the workload really crosses daughters beyond 4 m
    sin = st.cpu().numpy().view(vg.NAVSTATE_DTYPE)["nav_ind"]
    sout = res[0][0].view(vg.NAVSTATE_DTYPE)["nav_ind"]
    assert (sin != sout).mean() > 0.05
