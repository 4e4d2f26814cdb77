"""Spatio-temporal Markov GP models: MarkovVariationalGP with a
SpatioTemporalKernel (the reference's MarkovGaussianProcess in its
spatio-temporal case, basemodels.py:625-764, with the VI inference of
inference.py:160-222), stepped by libbnx.so.

    kern = SpatioTemporalMatern32(variance=1, lengthscale_time=10, lengthscale_space=0.3, z=z)
    model = MarkovVariationalGP(kern, Poisson(), X, Y, R=R)   # X [Nt], R [Nt, Nr, 2], Y [Nt, Nr]
    model.inference(lr=1.0)
    model.energy()

Every time point carries the same number Nr of observations (the reference's
input layout for spatio-temporal data).  posterior_mean / posterior_variance
are the latent marginals [Nt, M, 1] / [Nt, M, M] of u(t) = H x(t), as in the
reference; data_mean / data_variance are the marginals of f at the
observations.  Float32 on the device.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .cubature import GaussHermite


class STMarkovGaussianProcess:
    """Markov in time, sparse in space (M inducing inputs); VI sites in data space."""
    _method = _lib.METHOD_VI

    def __init__(self, kernel, likelihood, X, Y, R, parallel=None, dtype=torch.float32, device=None,
                 cubature=None):
        if dtype != torch.float32:
            raise NotImplementedError("the spatio-temporal path computes in float32")
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        self.dtype = dtype
        self.kernel = kernel
        self.likelihood = likelihood
        self.cubature = cubature or GaussHermite()
        self.parallel = True
        X = np.asarray(X, dtype=np.float64).reshape(-1)
        R = np.asarray(R, dtype=np.float64)
        Y = np.asarray(Y, dtype=np.float64)
        if R.ndim == 2:
            R = R[..., None]
        if Y.ndim != 2 or R.shape[:2] != Y.shape or X.shape[0] != Y.shape[0]:
            raise ValueError("expected X [Nt], R [Nt, Nr, D], Y [Nt, Nr]")
        ind = np.argsort(X, kind="stable")
        X, R, Y = X[ind], R[ind], Y[ind]
        if R.shape[2] != kernel.z.shape[1]:
            raise ValueError("R and z have different spatial dimensions")
        self.num_time, self.num_space = Y.shape
        self.M = kernel.M
        kw = dict(device=self.device, dtype=torch.float32)
        self.X = torch.as_tensor(X, **kw)
        self._t64 = torch.as_tensor(X, device=self.device, dtype=torch.float64).contiguous()
        self.R = torch.as_tensor(np.ascontiguousarray(R), **kw).contiguous()
        self.Y = torch.as_tensor(np.ascontiguousarray(Y), **kw).contiguous()
        self.dt = torch.as_tensor(np.concatenate([[0.0], np.diff(X)]), **kw).contiguous()
        n = self.num_time * self.num_space
        # sites start at mean 0, covariance 1e2 (basemodels.py:130-133)
        self._nat1 = torch.zeros(n, **kw)
        self._nat2 = torch.full((n,), 1e-2, **kw)
        self._pm = torch.zeros(n, **kw)
        self._pv = torch.ones(n, **kw)
        self._grad = torch.zeros(n, **kw)
        self._hess = torch.zeros(n, **kw)
        self._lin = torch.zeros(n, **kw)
        self._state = _lib.SiteState(self._nat1.data_ptr(), self._nat2.data_ptr(), self._pm.data_ptr(),
                                     self._pv.data_ptr(), self._grad.data_ptr(), self._hess.data_ptr(),
                                     self._lin.data_ptr())
        self._lib = _lib.load()
        self._handle = ctypes.c_void_p()
        self._desc = kernel.st_desc()
        _lib.check(self._lib.bn_st_create(ctypes.byref(self._desc), ctypes.byref(self._lik_desc()), self.num_time,
                                          self.num_space, ctypes.c_void_p(self.R.data_ptr()),
                                          ctypes.byref(self._handle)), "bn_st_create")
        self._versions = (kernel.version, likelihood.version)
        self._stale = True
        self._result = None
        self._post = None

    def _lik_desc(self):
        return self.likelihood.desc(self._method, self.cubature.num_cub_points, 1.0, True, False)

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _sync_params(self):
        v = (self.kernel.version, self.likelihood.version)
        if v != self._versions:
            self._desc = self.kernel.st_desc()
            _lib.check(self._lib.bn_st_set_prior(self._handle, ctypes.byref(self._desc)), "bn_st_set_prior")
            _lib.check(self._lib.bn_st_set_likelihood(self._handle, ctypes.byref(self._lik_desc())),
                       "bn_st_set_likelihood")
            self._versions = v
            self._stale = True

    def _fetch(self):
        if self._result is None:
            out = (ctypes.c_double * _lib.NRESULT)()
            st = ctypes.c_int32()
            _lib.check(self._lib.bn_st_result(self._handle, self._stream(), out, ctypes.byref(st)), "bn_st_result")
            self._result = (list(out), st.value)
        return self._result

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                self._lib.bn_st_destroy(h)
            except Exception:
                pass

    # ------------------------------------------------------------ reference API
    def update_posterior(self):
        self._sync_params()
        _lib.check(self._lib.bn_st_update_posterior(self._handle, self._stream(), self.dt.data_ptr(),
                                                    self.Y.data_ptr(), ctypes.byref(self._state)),
                   "bn_st_update_posterior")
        self._stale = False
        self._result = None
        self._post = None

    def inference(self, lr=1.0, **kwargs):
        self._sync_params()
        if self._stale:
            self.update_posterior()
        _lib.check(self._lib.bn_st_newton_step(self._handle, self._stream(), float(lr), self.dt.data_ptr(),
                                               self.Y.data_ptr(), ctypes.byref(self._state)), "bn_st_newton_step")
        self._result = None
        self._post = None

    def energy(self, **kwargs):
        self._sync_params()
        if self._stale:
            self.update_posterior()
        return self._fetch()[0][_lib.RES_ENERGY]

    def compute_log_lik(self):
        self._sync_params()
        if self._stale:
            self.update_posterior()
        return self._fetch()[0][_lib.RES_LOGLIK]

    def compute_kl(self):
        self._sync_params()
        if self._stale:
            self.update_posterior()
        res = self._fetch()[0]
        return res[_lib.RES_SUM2] - res[_lib.RES_LOGLIK]

    def status(self):
        return self._fetch()[1]

    def _latent(self):
        if self._post is None:
            m = torch.empty(self.num_time, self.M, device=self.device, dtype=torch.float32)
            P = torch.empty(self.num_time, self.M, self.M, device=self.device, dtype=torch.float32)
            _lib.check(self._lib.bn_st_latent_posterior(self._handle, self._stream(), ctypes.c_void_p(m.data_ptr()),
                                                        ctypes.c_void_p(P.data_ptr())), "bn_st_latent_posterior")
            self._post = (m, P)
        return self._post

    @property
    def posterior_mean(self):
        return self._latent()[0][..., None]

    @property
    def posterior_variance(self):
        return self._latent()[1]

    @property
    def data_mean(self):
        """Marginal means of f at the observations [Nt, Nr]."""
        return self._pm.view(self.num_time, self.num_space)

    @property
    def data_variance(self):
        return self._pv.view(self.num_time, self.num_space)

    def predict(self, X=None, R=None):
        """Posterior mean and variance of f at test times X [Nt*] and spatial inputs
        R [Nt*, Nr*, D] (basemodels.py:766-816): the state at each test time from
        its two neighbours' smoothed states, then the spatial conditional.  Returns
        ([Nt*, Nr*], [Nt*, Nr*]); X = None, R = None predict at the training inputs."""
        self._sync_params()
        if self._stale:
            self.update_posterior()
        self._fetch()
        if X is None:
            xt = self._t64
            Rt = self.R
        else:
            xt = torch.as_tensor(np.asarray(X, dtype=np.float64).reshape(-1), device=self.device)
            Rt = np.asarray(R, dtype=np.float32)
            if Rt.ndim == 2:
                Rt = Rt[..., None]
            if Rt.shape[0] != xt.shape[0] or Rt.shape[2] != self.kernel.z.shape[1]:
                raise ValueError("expected R [Nt*, Nr*, D] for X [Nt*]")
            Rt = torch.as_tensor(np.ascontiguousarray(Rt), device=self.device)
        nts, nrs = Rt.shape[0], Rt.shape[1]
        mean = torch.empty(nts, nrs, device=self.device, dtype=torch.float32)
        var = torch.empty(nts, nrs, device=self.device, dtype=torch.float32)
        _lib.check(self._lib.bn_st_predict(self._handle, self._stream(), self._t64.data_ptr(), nts, xt.data_ptr(),
                                           nrs, Rt.data_ptr(), mean.data_ptr(), var.data_ptr()), "bn_st_predict")
        return mean, var

    def set_profiling(self, on=True):
        _lib.check(self._lib.bn_st_set_profiling(self._handle, 1 if on else 0), "bn_st_set_profiling")

    def step_time(self):
        ms = ctypes.c_float()
        _lib.check(self._lib.bn_st_step_time(self._handle, ctypes.byref(ms)), "bn_st_step_time")
        return ms.value
