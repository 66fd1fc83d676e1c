"""Learned first-hit proposal for the BVH traversal (see include/vecgeom_gb300.h, "learned
proposal"): feature extraction, GPU training with the library's own forward/backward and
Adam kernels, inference, and attaching a trained model to a geometry so that steps with
NAV_LEARNED explore the proposed BVH subtree first."""
import ctypes

import numpy as np

from . import _check, _ptr, _stream, load_library

N_FEATURES = 80
N_CLASSES = 9
NAV_LEARNED = 8


def _lib():
    from . import _lib as lib
    if lib is None:
        load_library()
        from . import _lib as lib
    return lib


def features(geo, x, y, z, dx, dy, dz, states, labels=True):
    """80 FP32 features per track, the logical volume (-1: no proposal) and, optionally, the
    FP64 training label (0..7 subtree, 8 none, -1 n/a). CUDA tensors in, CUDA tensors out."""
    import torch
    n = x.numel()
    feat = torch.empty((n, N_FEATURES), dtype=torch.float32, device=x.device)
    lv = torch.empty(n, dtype=torch.int32, device=x.device)
    lab = torch.empty(n, dtype=torch.int8, device=x.device) if labels else None
    _check(_lib().vg_learn_features(geo._h, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy), _ptr(dz), _ptr(states), n,
                                    _ptr(feat), _ptr(lv), _ptr(lab), _stream()), "vg_learn_features")
    return feat, lv, lab


class Proposer:
    """The MLP of the learned proposal, on the device of `geo`."""

    def __init__(self, geo, seed=0):
        h = ctypes.c_void_p()
        _check(_lib().vg_mlp_create(geo._h, seed, ctypes.byref(h)), "vg_mlp_create")
        self._h = h
        self.n_params = int(_lib().vg_mlp_param_count(h))

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                _lib().vg_mlp_destroy(self._h)
                self._h = None
        except Exception:  # interpreter shutdown
            pass

    def get_params(self):
        out = np.empty(self.n_params, dtype=np.float32)
        _check(_lib().vg_mlp_get_params(self._h, out.ctypes.data, out.size), "vg_mlp_get_params")
        return out

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        _check(_lib().vg_mlp_set_params(self._h, p.ctypes.data, p.size), "vg_mlp_set_params")

    def gradients(self, feat, lv, label):
        """Mean cross-entropy gradients (flat parameter layout) and summed loss."""
        import torch
        g = torch.empty(self.n_params, dtype=torch.float32, device=feat.device)
        loss = torch.empty(1, dtype=torch.float32, device=feat.device)
        _check(_lib().vg_mlp_gradients(self._h, _ptr(feat), _ptr(lv), _ptr(label), lv.numel(), _ptr(g), _ptr(loss),
                                       _stream()), "vg_mlp_gradients")
        return g, float(loss.item())

    def train(self, feat, lv, label, epochs=8, batch=4096, lr=3e-3, seed=1):
        """Adam over shuffled mini-batches; returns the mean loss per epoch. Pass samples with
        lv >= 0 and 0 <= label <= 8; the proposal is meant to be trained on steps that hit a
        daughter (labels 0..7), since "none" gives the traversal nothing to start from."""
        out = np.zeros(max(epochs, 1), dtype=np.float32)
        _check(_lib().vg_mlp_train(self._h, _ptr(feat), _ptr(lv), _ptr(label), lv.numel(), epochs, batch, lr, seed,
                                   out.ctypes.data, _stream()), "vg_mlp_train")
        return out[:epochs].tolist()

    def infer(self, feat, lv, logits=False, tensor=False):
        """Proposals from features; tensor=True uses the tcgen05 kernel."""
        import torch
        n = lv.numel()
        slot = torch.empty(n, dtype=torch.int8, device=feat.device)
        lg = torch.empty((n, 16), dtype=torch.float32, device=feat.device) if logits else None
        _check(_lib().vg_mlp_infer(self._h, _ptr(feat), _ptr(lv), n, _ptr(slot), _ptr(lg), 1 if tensor else 0,
                                   _stream()), "vg_mlp_infer")
        return (slot, lg) if logits else slot

    def error(self):
        """Reads and clears the tensor-core kernels' time-out flag."""
        e = ctypes.c_int32()
        _check(_lib().vg_mlp_error(self._h, ctypes.byref(e)), "vg_mlp_error")
        return e.value

    def attach(self, geo, tensor=True):
        """Use this model for NAV_LEARNED steps on `geo` (tensor-core proposals by default)."""
        _check(_lib().vg_geom_set_proposer(geo._h, self._h), "vg_geom_set_proposer")
        _check(_lib().vg_nav_set_proposal_kernel(geo._h, 1 if tensor else 0), "vg_nav_set_proposal_kernel")
        geo._proposer = self  # keep the model alive while attached


def propose(geo, x, y, z, dx, dy, dz, states, tensor=True, out=None):
    """Proposals of the model attached to `geo` for step inputs (what NAV_LEARNED uses);
    tensor=True uses the tcgen05 kernel."""
    flags = 1 if tensor else 0
    import torch
    n = x.numel()
    slot = out if out is not None else torch.empty(n, dtype=torch.int8, device=x.device)
    _check(_lib().vg_nav_propose(geo._h, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy), _ptr(dz), _ptr(states), n,
                                 _ptr(slot), flags, _stream()), "vg_nav_propose")
    return slot
