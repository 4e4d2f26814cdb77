"""Infinite-horizon Markov GPs (the interface of bayesnewton/basemodels.py
InfiniteHorizonGaussianProcess :1257-1308 and the models.py classes
InfiniteHorizonVariationalGP :162, InfiniteHorizonExpectationPropagationGP :261,
InfiniteHorizonNewtonGP :315, InfiniteHorizonPosteriorLinearisationGP :388) on
libbnx.so's steady-state filter and smoother.

Equidistant times, one latent.  The step follows the reference's call sequence,
which matters because the Riccati recursions are warm-started from the previous
call: inference() = update_posterior, site update, update_posterior;
energy() runs a fresh filter for the log marginal (compute_kl).

    model = InfiniteHorizonVariationalGP(kernel, likelihood, X, Y, dare_iters=20)
    model.inference(lr=1.0)
    model.energy()
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .cubature import GaussHermite
from .models import PseudoLikelihood, input_admin


class InfiniteHorizonGaussianProcess:
    _method = _lib.METHOD_VI

    def __init__(self, kernel, likelihood, X, Y, R=None, dare_iters=20, parallel=None, power=1.0,
                 dtype=torch.float32, device=None, cubature=None, score_form=None):
        if R is not None:
            raise NotImplementedError("spatio-temporal inputs are not supported by the infinite-horizon path")
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        self.dtype = dtype
        self.kernel = kernel
        self.likelihood = likelihood
        self.power = float(power)
        self.cubature = cubature or GaussHermite()
        if score_form is None:
            score_form = dtype == torch.float64 or getattr(likelihood, "link", None) == "probit"
        self.score_form = bool(score_form)
        self.parallel = True if parallel is None else bool(parallel)
        self.dare_iters = int(dare_iters)
        self.X, self.Y, self.dt, t64 = input_admin(X, Y, self.device, dtype)
        dt64 = np.diff(t64.cpu().numpy())
        if dt64.shape[0] > 1 and np.max(np.abs(np.diff(dt64))) >= 1e-6:
            raise ValueError("time steps must be equidistant (basemodels.py:1269)")
        if dt64.shape[0] < 1:
            raise ValueError("the infinite-horizon model needs at least two time points (its step is dt[1])")
        self.dt_step = float(dt64[0])
        if self.Y.shape[1] != 1 or kernel.measurement_model().shape[0] != 1:
            raise NotImplementedError("the infinite-horizon path covers one latent")
        self.num_data = N = self.X.shape[0]
        self.heteroscedastic = bool(torch.isnan(self.Y).any()) or likelihood.kind() != _lib.LIK_GAUSSIAN
        kw = dict(device=self.device, dtype=dtype)
        self.site_dim = 1
        self._nat1 = torch.zeros(N, 1, **kw)
        self._nat2 = torch.full((N, 1, 1), 1e-2, **kw)
        self._pm = torch.zeros(N, 1, **kw)
        self._pv = torch.ones(N, 1, 1, **kw)
        self._grad = torch.zeros(N, 1, **kw)
        self._hess = torch.zeros(N, 1, 1, **kw)
        self._lin = torch.zeros(N, 1, **kw)
        self._state = _lib.SiteState(self._nat1.data_ptr(), self._nat2.data_ptr(), self._pm.data_ptr(),
                                     self._pv.data_ptr(), self._grad.data_ptr(), self._hess.data_ptr(),
                                     self._lin.data_ptr())
        self.pseudo_likelihood = PseudoLikelihood(self)
        self._lib = _lib.load()
        self._handle = ctypes.c_void_p()
        code = {torch.float32: _lib.DTYPE_F32, torch.float64: _lib.DTYPE_F64}[dtype]
        _lib.check(self._lib.bn_ih_create(ctypes.byref(kernel.desc()), ctypes.byref(self._lik_desc()), N, code,
                                          self.dare_iters, ctypes.byref(self._handle)), "bn_ih_create")
        self._versions = (kernel.version, likelihood.version)
        self._updated = False
        self._result = None

    def _lik_desc(self):
        return self.likelihood.desc(self._method, self.cubature.num_cub_points, self.power,
                                    self._method != _lib.METHOD_PL, self.score_form)

    def _sync_params(self):
        v = (self.kernel.version, self.likelihood.version)
        if v != self._versions:
            _lib.check(self._lib.bn_ih_set_prior(self._handle, ctypes.byref(self.kernel.desc())), "bn_ih_set_prior")
            _lib.check(self._lib.bn_ih_set_likelihood(self._handle, ctypes.byref(self._lik_desc())),
                       "bn_ih_set_likelihood")
            self._versions = v

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _fetch(self):
        if self._result is None:
            out = (ctypes.c_double * _lib.NRESULT)()
            st = ctypes.c_int32()
            _lib.check(self._lib.bn_ih_result(self._handle, self._stream(), out, ctypes.byref(st)), "bn_ih_result")
            self._result = (list(out), st.value)
        return self._result

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                self._lib.bn_ih_destroy(h)
            except Exception:
                pass

    @property
    def posterior_mean(self):
        return self._pm[..., None]

    @property
    def posterior_variance(self):
        return self._pv

    def update_posterior(self):
        """Steady-state filter + smoother from the current sites (advances both
        Riccati warm starts); also the site expectations at the new posterior."""
        self._sync_params()
        _lib.check(self._lib.bn_ih_update_posterior(self._handle, self._stream(), self.dt_step,
                                                    1 if self.heteroscedastic else 0, self.Y.data_ptr(),
                                                    ctypes.byref(self._state)), "bn_ih_update_posterior")
        self._updated = True
        self._result = None

    def inference(self, lr=1.0, **kwargs):
        """InferenceMixin.inference (inference.py:65-90)."""
        self.update_posterior()
        _lib.check(self._lib.bn_ih_site_update(self._handle, self._stream(), float(lr), ctypes.byref(self._state)),
                   "bn_ih_site_update")
        diffs = self._fetch()[0][_lib.RES_DIFF1:_lib.RES_DIFF2 + 1]
        self.update_posterior()
        return None, (diffs[0] / self.num_data, diffs[1] / self.num_data)

    def compute_log_lik(self):
        """The steady-state filter's log marginal of the pseudo-observations
        (advances the filter's Riccati warm start)."""
        self._sync_params()
        _lib.check(self._lib.bn_ih_log_lik(self._handle, self._stream(), self.dt_step,
                                           1 if self.heteroscedastic else 0, self.Y.data_ptr(),
                                           ctypes.byref(self._state)), "bn_ih_log_lik")
        self._result = None
        return self._fetch()[0][_lib.RES_LOGLIK]

    def energy(self, **kwargs):
        """The method's energy at the last posterior, with log Z from a fresh filter
        (compute_kl, basemodels.py:708-724)."""
        if not self._updated:
            self.update_posterior()
        self.compute_log_lik()
        return self._fetch()[0][_lib.RES_ENERGY]

    def status(self):
        return self._fetch()[1]

    def dare_state(self):
        """(filter, smoother) Riccati warm starts, [D, D] each."""
        D = self.kernel.state_dim
        f = (ctypes.c_double * (D * D))()
        s = (ctypes.c_double * (D * D))()
        _lib.check(self._lib.bn_ih_dare_state(self._handle, self._stream(), f, s), "bn_ih_dare_state")
        return np.array(f).reshape(D, D), np.array(s).reshape(D, D)


IHGP = InfiniteHorizonGaussianProcess


class InfiniteHorizonVariationalGP(InfiniteHorizonGaussianProcess):
    _method = _lib.METHOD_VI


class InfiniteHorizonNewtonGP(InfiniteHorizonGaussianProcess):
    _method = _lib.METHOD_NEWTON


class InfiniteHorizonExpectationPropagationGP(InfiniteHorizonGaussianProcess):
    _method = _lib.METHOD_EP


class InfiniteHorizonPosteriorLinearisationGP(InfiniteHorizonGaussianProcess):
    _method = _lib.METHOD_PL

    def __init__(self, *args, **kw):
        kw["power"] = 1.0
        super().__init__(*args, **kw)
