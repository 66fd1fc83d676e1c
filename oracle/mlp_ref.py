"""ORACLE — TEST INFRASTRUCTURE ONLY (the checker of the learned proposal; never shipped).

FP64 numpy restatement of the proposal MLP of vecgeom_gb300 (layout in
include/vecgeom_gb300.h, "learned proposal"): forward pass, softmax cross-entropy and its
gradients, used to check the library's GPU backward kernels; and the BF16 inference
semantics (inputs, hidden activations, weights and biases rounded to BF16, sums in
higher precision) used to check its inference kernels. The reference has no learned part,
so this is the only checker for it.
"""
import numpy as np

IN, HID, OUT, CLS, EMB, EOFF = 80, 64, 16, 9, 16, 6
W1 = 0
B1 = W1 + HID * IN
W2 = B1 + HID
B2 = W2 + HID * HID
W3 = B2 + HID
B3 = W3 + OUT * HID
E = B3 + OUT


def unpack(p, n_lv):
    p = np.asarray(p, dtype=np.float64)
    return dict(W1=p[W1:B1].reshape(HID, IN), b1=p[B1:W2], W2=p[W2:B2].reshape(HID, HID), b2=p[B2:W3],
                W3=p[W3:B3].reshape(OUT, HID), b3=p[B3:E], E=p[E:E + n_lv * EMB].reshape(n_lv, EMB))


def gradients(params, n_lv, feat, lv, label):
    """Mean cross-entropy gradients (flat layout, float64) and the summed loss."""
    w = unpack(params, n_lv)
    n = len(lv)
    X = np.asarray(feat, dtype=np.float64).copy()
    X[:, EOFF:EOFF + EMB] = w["E"][lv]
    Z1 = X @ w["W1"].T + w["b1"]
    H1 = np.maximum(Z1, 0)
    Z2 = H1 @ w["W2"].T + w["b2"]
    H2 = np.maximum(Z2, 0)
    Z3 = H2 @ w["W3"].T + w["b3"]
    L = Z3[:, :CLS]
    mx = L.max(axis=1, keepdims=True)
    lse = mx[:, 0] + np.log(np.exp(L - mx).sum(axis=1))
    y = np.asarray(label, dtype=np.int64)
    loss = float((lse - L[np.arange(n), y]).sum())
    P = np.exp(L - lse[:, None])
    dZ3 = np.zeros_like(Z3)
    dZ3[:, :CLS] = P
    dZ3[np.arange(n), y] -= 1.0
    dZ3 /= n
    g = np.zeros(E + n_lv * EMB)
    g[W3:B3] = (dZ3.T @ H2).ravel()
    g[B3:E] = dZ3.sum(0)
    dZ2 = (dZ3 @ w["W3"]) * (Z2 > 0)
    g[W2:B2] = (dZ2.T @ H1).ravel()
    g[B2:W3] = dZ2.sum(0)
    dZ1 = (dZ2 @ w["W2"]) * (Z1 > 0)
    g[W1:B1] = (dZ1.T @ X).ravel()
    g[B1:W2] = dZ1.sum(0)
    dX = dZ1 @ w["W1"]
    dE = np.zeros((n_lv, EMB))
    np.add.at(dE, np.asarray(lv), dX[:, EOFF:EOFF + EMB])
    g[E:] = dE.ravel()
    return g, loss


def bf16(x):
    """Round float32 values to BF16 (nearest, ties to even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def infer_logits(params, n_lv, feat, lv):
    """Logits under the BF16 inference semantics (float64 sums of BF16 products)."""
    w = {k: bf16(v.astype(np.float32)).astype(np.float64) for k, v in unpack(params, n_lv).items()}
    X = bf16(np.asarray(feat, dtype=np.float32)).astype(np.float64)
    X[:, EOFF:EOFF + EMB] = w["E"][lv]
    H1 = bf16(np.maximum(X @ w["W1"].T + w["b1"], 0).astype(np.float32)).astype(np.float64)
    H2 = bf16(np.maximum(H1 @ w["W2"].T + w["b2"], 0).astype(np.float32)).astype(np.float64)
    return (H2 @ w["W3"].T + w["b3"])[:, :CLS]
