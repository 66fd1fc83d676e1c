"""CUDA-graph replay of the scheduled step: one call of the sorted, learned, work-queue step
(sort, tensor-core proposals, persistent step kernel) captured into a graph and replayed
gives the eager call's states and steps, also after the inputs change in place; the plain
FP64 step likewise."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def detector(cuda):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import learned as L
    from vecgeom_gb300 import workloads as W
    g = vg.Geometry()
    W.build_detector(g)
    model = L.Proposer(g, seed=5)
    model.attach(g)
    return g, model


def _inputs(cuda, g, n, seed):
    from vecgeom_gb300 import workloads as W
    t, st, _ = W.sample_transport_steps(g, n, seed, cuda, "cuda:0", n_primaries=1 << 14)
    return t, st


@pytest.mark.parametrize("flags_name", ["learned", "fp64"])
def test_graph_replay_matches_eager(cuda, detector, flags_name):
    import vecgeom_gb300 as vg
    g, model = detector
    flags = (vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE | vg.NAV_LEARNED) if flags_name == "learned" else vg.PREC_FP64
    n = (1 << 16) + 77
    t, st = _inputs(cuda, g, n, 41)
    out_e = cuda.empty_like(st)
    step_e = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
    g.compute_step_and_next_volume(*t, st, out_e, step_e, flags=flags)

    ws = cuda.empty(max(vg.Geometry.step_workspace_bytes(n, flags), 256), dtype=cuda.uint8, device="cuda:0")
    out_g = cuda.zeros_like(st)
    step_g = cuda.zeros(n, dtype=cuda.float64, device="cuda:0")
    side = cuda.cuda.Stream()
    side.wait_stream(cuda.cuda.current_stream())
    with cuda.cuda.stream(side):  # warm-up outside the capture (one-time kernel setup)
        g.compute_step_and_next_volume(*t, st, out_g, step_g, flags=flags, workspace=ws)
    cuda.cuda.current_stream().wait_stream(side)
    graph = cuda.cuda.CUDAGraph()
    with cuda.cuda.graph(graph):
        g.compute_step_and_next_volume(*t, st, out_g, step_g, flags=flags, workspace=ws)
    out_g.zero_()
    step_g.zero_()
    graph.replay()
    cuda.cuda.synchronize()
    assert cuda.equal(out_g, out_e)
    assert cuda.equal(step_g, step_e)

    # new inputs copied into the captured buffers: the replay follows them
    t2, st2 = _inputs(cuda, g, n, 42)
    for a, b in zip(t, t2):
        a.copy_(b)
    st.copy_(st2)
    g.compute_step_and_next_volume(*t, st, out_e, step_e, flags=flags)
    graph.replay()
    cuda.cuda.synchronize()
    assert cuda.equal(out_g, out_e)
    assert cuda.equal(step_g, step_e)
    assert model.error() == 0
    assert int((step_e > 0).sum().item()) > n // 2


def test_pipelined_host_entry_matches_device(cuda, detector):
    """The host-pointer step with a sorted schedule copies its inputs in chunks that overlap
    the sort keys and proposals of the chunks already arrived; the result equals the
    device-pointer call."""
    import vecgeom_gb300 as vg
    g, model = detector
    flags = vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE | vg.NAV_LEARNED
    n = (1 << 18) + 77
    t, st = _inputs(cuda, g, n, 43)
    out_d = cuda.empty_like(st)
    step_d = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
    g.compute_step_and_next_volume(*t, st, out_d, step_d, flags=flags)
    h = [a.cpu().pin_memory() for a in t]
    sh = st.cpu().pin_memory()
    out_h = cuda.empty(n * 12, dtype=cuda.uint8).pin_memory()
    step_h = cuda.empty(n, dtype=cuda.float64).pin_memory()
    status_h = cuda.empty(n, dtype=cuda.int32).pin_memory()
    for _ in range(2):  # the second call reuses the staging buffers and copy stream
        g.compute_step_and_next_volume_host(*h, sh, out_h, step_h, status=status_h, flags=flags)
        assert cuda.equal(out_h, out_d.cpu())
        assert cuda.equal(step_h, step_d.cpu())
        assert int(status_h.abs().sum().item()) == 0
    assert model.error() == 0
