"""The benchmark's step inputs (straight-track transport histories generated on the GPU by
the FP64 navigator, a seeded draw of pre-step points) equal their reproduction on the CPU by
the oracle, bit for bit: every position, direction and state of the draw. This is what lets
the CPU baseline and the CPU reference arm step exactly the GPU arm's inputs, and it checks
the GPU's FP64 transport against the oracle over whole track histories."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("workload", ["barrel", "detector"])
def test_transport_sample_reproduced_on_cpu(cuda, workload):
    import vecgeom_gb300 as vg
    from oracle.oracle import NAVSTATE_DTYPE, OracleGeometry, transport_step_sample
    from vecgeom_gb300 import workloads as W
    build = W.build_detector if workload == "detector" else W.build_barrel
    g = vg.Geometry()
    build(g)
    o = OracleGeometry()
    build(o)
    n_samples, n_primaries, seed = 20_000, 4096, 0xC0FFEE
    t, st, total = W.sample_transport_steps(g, n_samples, seed, cuda, cuda.device("cuda", 0),
                                            n_primaries=n_primaries)
    cols, ost, ototal = transport_step_sample(o, n_samples, seed, n_primaries, nthreads=os.cpu_count() or 1)
    assert total == ototal
    for a, b in zip(t, cols):
        assert np.array_equal(a.cpu().numpy().view(np.int64), b.view(np.int64))
    gst = np.frombuffer(st.cpu().numpy().tobytes(), dtype=NAVSTATE_DTYPE)
    for f in ("nav_ind", "last_exited", "on_boundary"):
        assert np.array_equal(gst[f], ost[f]), f
    # the leading samples alone (what the reference arm uses)
    c2, s2, _ = transport_step_sample(o, n_samples, seed, n_primaries, nthreads=os.cpu_count() or 1, first=512)
    assert np.array_equal(c2[0], cols[0][:512]) and np.array_equal(s2["nav_ind"], ost["nav_ind"][:512])
