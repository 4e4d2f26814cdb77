"""Learned site expectations for the two-latent heteroscedastic likelihood.

A 6-64-64-64-6 tanh network maps a site's (y, m1, m2, v11, v12, v22) to
(E, dE/dm, d2E/dm2) of E_q log p(y | f), the quantity the reference integrates
with 2-D Gauss-Hermite cubature (likelihoods.py:613-664).  Training pairs come
from high-order cubature on the device; training (forward, backward, Adam) runs
in libbnx.so's own kernels.

    sur = CubatureSurrogate(likelihood)
    sur.fit(model.site_inputs(augment=4))        # cubature-generated pairs
    model.set_surrogate(sur, spot=64, tol=0.05)  # the model's sites use it
    model.inference(lr=0.5); model.surrogate_counts()

Cubature stays the fallback and the reference value: sites whose predicted diagonal
precision (-h11, -h22) is not positive, and spot-checked sites whose prediction
misses the cubature by more than tol, are integrated by cubature in that step
(counted per step).
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


class CubatureSurrogate:
    def __init__(self, likelihood, device=None, seed=0):
        kind = likelihood.kind()
        if kind not in (_lib.LIK_HETERO_EXP, _lib.LIK_HETERO_SOFTPLUS):
            raise NotImplementedError("the learned sites cover the HeteroscedasticNoise likelihood")
        self.kind = kind
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        _lib.check(self._lib.bn_mlp_create(kind, ctypes.byref(self._h)), "bn_mlp_create")
        self.num_params = int(self._lib.bn_mlp_num_params())
        self.init_params(seed)
        self.history = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.bn_mlp_destroy(h)
            except Exception:
                pass

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    # ------------------------------------------------------------ parameters
    def init_params(self, seed=0):
        """Glorot-uniform weights, zero biases, identity standardisation."""
        rng = np.random.default_rng(seed)
        parts = []
        for fan_out, fan_in in ((64, 6), (64, 64), (64, 64), (6, 64)):
            a = math.sqrt(6.0 / (fan_in + fan_out))
            parts.append(rng.uniform(-a, a, fan_out * fan_in))
            parts.append(np.zeros(fan_out))
        self.set_params(np.concatenate(parts), np.concatenate([np.zeros(6), np.ones(6), np.zeros(6), np.ones(6)]))

    def set_params(self, params=None, norm=None):
        fp = ctypes.POINTER(ctypes.c_float)
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        _lib.check(self._lib.bn_mlp_set_params(self._h, None if p is None else p.ctypes.data_as(fp),
                                               None if n is None else n.ctypes.data_as(fp)), "bn_mlp_set_params")

    def get_params(self):
        p = np.zeros(self.num_params, dtype=np.float32)
        n = np.zeros(24, dtype=np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        _lib.check(self._lib.bn_mlp_get_params(self._h, p.ctypes.data_as(fp), n.ctypes.data_as(fp)),
                   "bn_mlp_get_params")
        return p, n

    # ------------------------------------------------------------ data
    def _link(self, m2):
        return torch.exp(m2) if self.kind == _lib.LIK_HETERO_EXP else torch.nn.functional.softplus(m2)

    def prepare(self, raw, ncub=32, targets=True):
        """raw [n, 6] (device float32) -> (xn, tn, traw): standardised features and,
        from ncub x ncub Gauss-Hermite cubature, standardised and raw targets."""
        raw = raw.to(self.device, torch.float32).contiguous()
        n = raw.shape[0]
        xn = torch.empty_like(raw)
        tn = torch.empty_like(raw) if targets else None
        traw = torch.empty_like(raw) if targets else None
        _lib.check(self._lib.bn_mlp_prepare(self._h, self._stream(), n, ncub, _vp(raw), _vp(xn),
                                            None if tn is None else _vp(tn), None if traw is None else _vp(traw)),
                   "bn_mlp_prepare")
        return xn, tn, traw

    def _scaled(self, raw, traw):
        l = self._link(raw[:, 2])
        return torch.stack([traw[:, 0] + torch.log(l), traw[:, 1] * l, traw[:, 2], traw[:, 3] * l * l,
                            traw[:, 4] * l, traw[:, 5]], 1)

    # ------------------------------------------------------------ training
    def fit(self, raw, ncub=32, steps=2000, batch=4096, lr=2e-3, seed=0):
        """Standardise on the training inputs, generate cubature targets, train
        with Adam.  Returns the loss of the last mini-batch (standardised units)."""
        raw = raw.to(self.device, torch.float32).contiguous()
        p, _ = self.get_params()
        self.set_params(None, np.concatenate([np.zeros(6), np.ones(6), np.zeros(6), np.ones(6)]))
        xr, _, traw = self.prepare(raw, ncub)
        s = self._scaled(raw, traw)
        ok = torch.isfinite(s).all(1) & torch.isfinite(xr).all(1)
        raw, xr, s = raw[ok].contiguous(), xr[ok], s[ok]
        norm = torch.cat([xr.mean(0), xr.std(0).clamp_min(1e-6), s.mean(0), s.std(0).clamp_min(1e-6)])
        self.set_params(p, norm.cpu().numpy())
        xn, tn, _ = self.prepare(raw, ncub)
        loss = ctypes.c_double()
        # three phases of a step-decayed learning rate (lr, lr / 4, lr / 16)
        for i, f in enumerate((1.0, 0.25, 0.0625)):
            _lib.check(self._lib.bn_mlp_train(self._h, self._stream(), xn.shape[0], _vp(xn), _vp(tn),
                                              max(1, int(steps) // 3), int(batch), float(lr * f),
                                              (int(seed) + 7919 * i) & 0xFFFFFFFF, ctypes.byref(loss)),
                       "bn_mlp_train")
            self.history.append(loss.value)
        return loss.value

    def loss_grad(self, xn, tn):
        """(loss, gradient as numpy) on standardised device tensors."""
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = ctypes.c_double()
        _lib.check(self._lib.bn_mlp_loss_grad(self._h, self._stream(), xn.shape[0], _vp(xn), _vp(tn),
                                              ctypes.byref(loss), g.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
                   "bn_mlp_loss_grad")
        return loss.value, g

    def forward(self, xn):
        out = torch.empty_like(xn)
        _lib.check(self._lib.bn_mlp_forward(self._h, self._stream(), xn.shape[0], _vp(xn), _vp(out)),
                   "bn_mlp_forward")
        return out

    def predict(self, raw):
        """(E, g1, g2, h11, h12, h22) [n, 6] for raw sites [n, 6]."""
        raw = raw.to(self.device, torch.float32).contiguous()
        xn, _, _ = self.prepare(raw, targets=False)
        o = self.forward(xn)
        _, norm = self.get_params()
        norm = torch.as_tensor(norm, device=self.device)
        s = o * norm[18:24] + norm[12:18]
        l = self._link(raw[:, 2])
        return torch.stack([s[:, 0] - torch.log(l), s[:, 1] / l, s[:, 2], s[:, 3] / (l * l), s[:, 4] / l, s[:, 5]], 1)
