"""The FP64 numpy checker of the learned proposal (oracle/mlp_ref.py) against central
finite differences, so that it can in turn check the GPU backward kernels."""
import numpy as np

from oracle import mlp_ref as M


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(5)
    n_lv, n = 3, 7
    p = rng.normal(0, 0.3, M.E + n_lv * M.EMB)
    feat = rng.normal(0, 1, (n, M.IN))
    lv = rng.integers(0, n_lv, n)
    y = rng.integers(0, M.CLS, n)
    g, _ = M.gradients(p, n_lv, feat, lv, y)
    idx = np.concatenate([rng.choice(np.arange(b, e), min(12, e - b), replace=False) for b, e in
                          [(M.W1, M.B1), (M.B1, M.W2), (M.W2, M.B2), (M.B2, M.W3), (M.W3, M.B3), (M.B3, M.B3 + M.CLS),
                           (M.E, M.E + n_lv * M.EMB)]])
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp = M.gradients(q, n_lv, feat, lv, y)[1]
        q[i] -= 2 * h
        lm = M.gradients(q, n_lv, feat, lv, y)[1]
        fd = (lp - lm) / (2 * h) / n
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-39], dtype=np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # 1 + 2^-8 is a tie: rounds to the even mantissa
    assert r[2] == np.float32(1.0078125)
    assert r[3] == -2.5
