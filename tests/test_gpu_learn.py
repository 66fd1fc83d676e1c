"""Learned first-hit proposal on the GPU: features and FP64 labels, gradients of the
library's backward kernels against the FP64 numpy checker (oracle/mlp_ref.py), training,
BF16 inference against the checker, and the learned step: identical results to the step
without the proposal and fewer BVH nodes visited."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def barrel(cuda):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import learned as L
    from vecgeom_gb300 import workloads as W
    g = vg.Geometry()
    W.build_barrel(g)
    dev = cuda.device("cuda", 0)
    t, st, _ = W.sample_transport_steps(g, 1 << 19, 2024, cuda, dev, n_primaries=1 << 16)
    feat, lv, lab = L.features(g, *t, st)
    return g, t, st, feat, lv, lab


def _valid(lv, lab, hits_only=False):
    return ((lv >= 0) & (lab >= 0) & (lab <= (7 if hits_only else 8))).nonzero().flatten()


def test_features_and_labels(cuda, barrel):
    import vecgeom_gb300 as vg
    g, t, st, feat, lv, lab = barrel
    lvh, labh = lv.cpu().numpy(), lab.cpu().numpy()
    assert (lvh >= 0).mean() > 0.2
    assert (labh[lvh < 0] == -1).all()
    assert ((labh >= -1) & (labh <= 8)).all()
    assert np.isfinite(feat.cpu().numpy()).all()
    # label semantics against the FP64 step: 0..7 means the step enters a daughter, 8 not
    n = lv.numel()
    out = cuda.empty_like(st)
    step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
    g.compute_step_and_next_volume(*t, st, out, step, flags=vg.PREC_FP64)
    nav = g.nav_table().astype(np.int64)
    sin = st.cpu().numpy().view(vg.NAVSTATE_DTYPE)["nav_ind"].astype(np.int64)
    sout = out.cpu().numpy().view(vg.NAVSTATE_DTYPE)["nav_ind"].astype(np.int64)
    lvl_in = nav[sin + 2] & 0xFF
    lvl_out = np.where(sout > 0, nav[np.maximum(sout, 1) + 2] & 0xFF, -1)
    sel = lvh >= 0
    entered = lvl_out > lvl_in
    assert (entered[sel & (labh >= 0) & (labh < 8)]).all()
    # no daughter hit: the step leaves the volume (relocation could only enter a volume
    # that touches the exit point)
    assert entered[sel & (labh == 8)].mean() < 1e-3


def test_gradients_match_fp64_checker(cuda, barrel):
    from oracle import mlp_ref as M
    from vecgeom_gb300 import learned as L
    g, t, st, feat, lv, lab = barrel
    idx = _valid(lv, lab)[:512]
    f, l, y = feat[idx].contiguous(), lv[idx].contiguous(), lab[idx].contiguous()
    model = L.Proposer(g, seed=3)
    n_lv = g.info()["n_lv"]
    rng = np.random.default_rng(11)
    p = rng.normal(0, 0.2, model.n_params).astype(np.float32)
    model.set_params(p)
    grads, loss = model.gradients(f, l, y)
    ref, ref_loss = M.gradients(p.astype(np.float64), n_lv, f.cpu().numpy(), l.cpu().numpy(), y.cpu().numpy())
    got = grads.cpu().numpy().astype(np.float64)
    assert abs(loss - ref_loss) <= 1e-4 * abs(ref_loss)
    for name, (b, e) in {"W1": (M.W1, M.B1), "b1": (M.B1, M.W2), "W2": (M.W2, M.B2), "b2": (M.B2, M.W3),
                         "W3": (M.W3, M.B3), "b3": (M.B3, M.E), "E": (M.E, M.E + n_lv * M.EMB)}.items():
        err = np.linalg.norm(got[b:e] - ref[b:e]) / max(np.linalg.norm(ref[b:e]), 1e-30)
        assert err < 1e-4, (name, err)


@pytest.fixture(scope="module")
def trained(cuda, barrel):
    from vecgeom_gb300 import learned as L
    g, t, st, feat, lv, lab = barrel
    idx = _valid(lv, lab, hits_only=True)  # the proposal is trained on steps that hit a daughter
    n = idx.numel()
    tr, te = idx[: n * 3 // 4], idx[n * 3 // 4:]
    model = L.Proposer(g, seed=7)
    losses = model.train(feat[tr].contiguous(), lv[tr].contiguous(), lab[tr].contiguous(), epochs=8, batch=4096,
                         lr=3e-3, seed=5)
    return model, losses, te


def test_training_learns(cuda, barrel, trained):
    g, t, st, feat, lv, lab = barrel
    model, losses, te = trained
    assert losses[-1] < 0.8 * losses[0], losses
    slot = model.infer(feat[te].contiguous(), lv[te].contiguous()).cpu().numpy().astype(np.int64)
    y = lab[te].cpu().numpy().astype(np.int64)  # held-out steps that hit a daughter
    acc = (slot == y).mean()
    majority = np.bincount(y, minlength=9).max() / len(y)
    assert acc > max(0.5, majority + 0.2), (acc, majority)


def test_simt_inference_matches_bf16_checker(cuda, barrel, trained):
    from oracle import mlp_ref as M
    g, t, st, feat, lv, lab = barrel
    model, _, te = trained
    sel = te[:4096]
    f, l = feat[sel].contiguous(), lv[sel].contiguous()
    slot, logits = model.infer(f, l, logits=True)
    ref = M.infer_logits(model.get_params(), g.info()["n_lv"], f.cpu().numpy(), l.cpu().numpy())
    got = logits.cpu().numpy()[:, :M.CLS].astype(np.float64)
    # FP32 vs FP64 sums: a hidden activation next to a BF16 rounding boundary may round to
    # the neighbouring BF16 value, so a few logits move by up to ~2^-8 relative
    d, scale = np.abs(got - ref), max(1.0, np.abs(ref).max())
    assert (d <= 1e-5 * scale).mean() > 0.99
    assert d.max() <= 1e-2 * scale
    s = np.sort(ref, axis=1)
    clear = (s[:, -1] - s[:, -2]) > 0.1
    refslot = np.argmax(ref, axis=1)
    refslot = np.where(refslot == 8, -1, refslot)
    assert (slot.cpu().numpy()[clear] == refslot[clear]).all()


def test_learned_step_identical_and_visits_fewer_nodes(cuda, barrel, trained):
    import vecgeom_gb300 as vg
    g, t, st, feat, lv, lab = barrel
    model, _, te = trained
    model.attach(g)
    n = lv.numel()

    def run(flags):
        out = cuda.empty_like(st)
        step = cuda.empty(n, dtype=cuda.float64, device="cuda:0")
        nodes = cuda.empty(n, dtype=cuda.int32, device="cuda:0")
        g.compute_step_and_next_volume(*t, st, out, step, flags=flags, nodes_visited=nodes)
        return out.cpu().numpy(), step.cpu().numpy(), nodes.cpu().numpy()

    base = vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE
    o0, s0, n0 = run(base)
    o1, s1, n1 = run(base | vg.NAV_LEARNED)
    assert np.array_equal(o0, o1)
    assert np.array_equal(s0, s1)
    held = te.cpu().numpy()
    assert n1[held].mean() < n0[held].mean(), (n1[held].mean(), n0[held].mean())


def test_tensor_core_inference_matches_simt(cuda, barrel, trained):
    """tcgen05 inference (BF16 operands in shared memory, FP32 accumulator in tensor memory)
    against the SIMT kernel on the same features. The two sum in different orders, so a
    hidden activation next to a BF16 rounding boundary can round to the neighbouring BF16
    value (a 2^-8 relative step) and move the logits slightly: nearly all logits agree to
    FP32 rounding, all within 1% of the logit range, and the proposals agree wherever the
    top two logits are 0.1 apart."""
    g, t, st, feat, lv, lab = barrel
    model, _, te = trained
    sel = te[: (1 << 15) + 77]  # a ragged last tile
    f, l = feat[sel].contiguous(), lv[sel].contiguous()
    s0, l0 = model.infer(f, l, logits=True)
    s1, l1 = model.infer(f, l, logits=True, tensor=True)
    assert model.error() == 0
    a, b = l0.cpu().numpy()[:, :9], l1.cpu().numpy()[:, :9]
    d = np.abs(a - b)
    scale = max(1.0, np.abs(a).max())
    assert (d <= 1e-5 * scale).mean() > 0.99, (d <= 1e-5 * scale).mean()
    assert d.max() <= 1e-2 * scale, d.max()
    srt = np.sort(a, axis=1)
    clear = (srt[:, -1] - srt[:, -2]) > 0.1
    assert (s0.cpu().numpy()[clear] == s1.cpu().numpy()[clear]).all()


def test_tensor_core_propose_matches_simt(cuda, barrel, trained):
    from vecgeom_gb300 import learned as L
    g, t, st, feat, lv, lab = barrel
    model, _, te = trained
    model.attach(g)
    p0 = L.propose(g, *t, st, tensor=False).cpu().numpy()
    p1 = L.propose(g, *t, st, tensor=True).cpu().numpy()
    assert model.error() == 0
    assert (p0 == p1).mean() > 0.999
    assert ((p0 == -1) == (lv.cpu().numpy() < 0)).all() or (p0[lv.cpu().numpy() < 0] == -1).all()
