"""Markov GP models (the interface of bayesnewton/models.py and
basemodels.MarkovGaussianProcess) whose inference step runs in libbnx.so.

    model = MarkovVariationalGP(kernel, likelihood, X, Y)
    for i in range(iters):
        model.inference(lr=1.0)        # site update + filter + smoother + energy terms
        energy = model.energy()        # negative ELBO at the current posterior

The model state (sites, posterior marginals and the site expectations at the
posterior) lives in torch CUDA tensors owned by the model; one C-ABI call runs a
whole step.  The reference recomputes the posterior at the start of every
inference() (inference.py:70); here it is kept current, and recomputed only when
a hyperparameter of the kernel or likelihood changed since it was computed.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from .cubature import GaussHermite
from .kernels import Independent, Sum


def input_admin(X, Y, device, dtype):
    """Sort by time and form dt = [0, diff(t)] (utils.py:234-265, temporal case)."""
    X = torch.as_tensor(np.asarray(X) if not isinstance(X, torch.Tensor) else X)
    Y = torch.as_tensor(np.asarray(Y) if not isinstance(Y, torch.Tensor) else Y)
    X = X.to(device=device, dtype=torch.float64)
    Y = Y.to(device=device, dtype=torch.float64)
    if X.ndim < 2:
        X = X[:, None]
    if Y.ndim < 2:
        Y = Y[:, None]
    if X.shape[1] > 1:
        raise NotImplementedError("spatial inputs are not supported by the temporal path")
    if X.shape[0] == 0 or X.shape[0] != Y.shape[0]:
        raise ValueError("X and Y need the same number (>= 1) of rows, got %d and %d" % (X.shape[0], Y.shape[0]))
    if not bool(torch.isfinite(X).all()):
        raise ValueError("X holds non-finite times (missing observations are NaN in Y, not in X)")
    t, ind = torch.sort(X[:, 0], stable=True)
    Y = Y[ind]
    dt = torch.cat([torch.zeros(1, device=device, dtype=torch.float64), t[1:] - t[:-1]])
    return t[:, None].to(dtype), Y.to(dtype).contiguous(), dt.to(dtype).contiguous(), t.contiguous()


class PseudoLikelihood:
    """Site parameters (basemodels.GaussianDistribution, :52-100): nat2 is the
    precision, nat1 = nat2 @ mean."""

    def __init__(self, model):
        self._m = model

    @property
    def nat1(self):
        return self._m._nat1[..., None]

    @property
    def nat2(self):
        return self._m._nat2

    @property
    def covariance(self):
        return torch.linalg.inv(self._m._nat2)

    @property
    def mean(self):
        return self.covariance @ self._m._nat1[..., None]

    def update_nat_params(self, nat1, nat2):
        self._m._nat1.copy_(nat1.reshape(self._m._nat1.shape))
        self._m._nat2.copy_(nat2.reshape(self._m._nat2.shape))
        self._m._stale = True


class MarkovGaussianProcess:
    """Markov GP on one sorted time series (basemodels.py:625-764).  With a
    SpatioTemporalKernel and spatial inputs R the model is the spatio-temporal
    one (bayesnewton_gb300.spatiotemporal)."""
    _method = _lib.METHOD_VI

    def __new__(cls, kernel=None, likelihood=None, X=None, Y=None, R=None, *args, **kw):
        from .kernels import SpatioTemporalKernel
        if R is not None and isinstance(kernel, SpatioTemporalKernel):
            from .spatiotemporal import STMarkovGaussianProcess
            if cls._method != _lib.METHOD_VI:
                raise NotImplementedError("the spatio-temporal path runs variational inference")
            kw.pop("power", None)
            return STMarkovGaussianProcess(kernel, likelihood, X, Y, R, *args, **kw)
        return super().__new__(cls)

    def __init__(self, kernel, likelihood, X, Y, R=None, parallel=None, power=1.0, dtype=torch.float32,
                 device=None, cubature=None, steps_per_thread=0, score_form=None):
        if R is not None:
            raise NotImplementedError("spatio-temporal inputs are not supported by the temporal path")
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        self.dtype = dtype
        self.kernel = kernel
        self.likelihood = likelihood
        self.power = float(power)
        self.cubature = cubature or GaussHermite()
        # the reference's score-form cubature derivatives (cubature.py:198-246) in
        # float64 and for the probit link; float32 logit sites use the derivative
        # expectations, which agree with them to ~1e-6 and round far less
        if score_form is None:
            score_form = dtype == torch.float64 or getattr(likelihood, "link", None) == "probit"
        self.score_form = bool(score_form)
        # parallel=None: the reference picks the scan on a GPU backend (basemodels.py:642-643)
        self.parallel = True if parallel is None else bool(parallel)
        self.X, self.Y, self.dt, self._t64 = input_admin(X, Y, self.device, dtype)
        self.num_data = self.X.shape[0]
        self.obs_dim = self.Y.shape[1]
        H = kernel.measurement_model()
        self.func_dim = H.shape[0]
        self.state_dim = kernel.state_dim
        P = self.func_dim if (isinstance(kernel, Independent) and not isinstance(kernel, Sum)) else self.obs_dim
        if P != self.func_dim:
            raise NotImplementedError("site dimension %d != latent dimension %d" % (P, self.func_dim))
        self.site_dim = P
        N = self.num_data
        kw = dict(device=self.device, dtype=dtype)
        # sites start at mean 0, covariance 1e2 I (basemodels.py:130-133)
        self._nat1 = torch.zeros(N, P, **kw)
        self._nat2 = (1e-2 * torch.eye(P, **kw)).repeat(N, 1, 1).contiguous()
        self._pm = torch.zeros(N, P, **kw)
        self._pv = torch.eye(P, **kw).repeat(N, 1, 1).contiguous()
        self._grad = torch.zeros(N, P, **kw)
        self._hess = torch.zeros(N, P, P, **kw)
        self._lin = torch.zeros(N, P, **kw)
        self._state = _lib.SiteState(self._nat1.data_ptr(), self._nat2.data_ptr(), self._pm.data_ptr(),
                                     self._pv.data_ptr(), self._grad.data_ptr(), self._hess.data_ptr(),
                                     self._lin.data_ptr())
        self.pseudo_likelihood = PseudoLikelihood(self)
        self._lib = _lib.load()
        self._handle = ctypes.c_void_p()
        code = {torch.float32: _lib.DTYPE_F32, torch.float64: _lib.DTYPE_F64}[dtype]
        _lib.check(self._lib.bn_model_create(ctypes.byref(kernel.desc()), ctypes.byref(self._lik_desc()), N,
                                             self.obs_dim, code, int(steps_per_thread),
                                             ctypes.byref(self._handle)), "bn_model_create")
        self._versions = self._param_versions()
        self._stale = True
        self._result = None

    # ------------------------------------------------------------ plumbing
    def _lik_desc(self):
        return self.likelihood.desc(self._method, self.cubature.num_cub_points, self.power, True, self.score_form)

    def _param_versions(self):
        return (self.kernel.version, self.likelihood.version)

    def _sync_params(self):
        v = self._param_versions()
        if v != self._versions:
            _lib.check(self._lib.bn_model_set_prior(self._handle, ctypes.byref(self.kernel.desc())),
                       "bn_model_set_prior")
            _lib.check(self._lib.bn_model_set_likelihood(self._handle, ctypes.byref(self._lik_desc())),
                       "bn_model_set_likelihood")
            self._versions = v
            self._stale = True

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _fetch(self):
        if self._result is None:
            out = (ctypes.c_double * _lib.NRESULT)()
            st = ctypes.c_int32()
            _lib.check(self._lib.bn_model_result(self._handle, self._stream(), out, ctypes.byref(st)),
                       "bn_model_result")
            self._result = (list(out), st.value)
        return self._result

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                self._lib.bn_model_destroy(h)
            except Exception:
                pass

    # ------------------------------------------------------------ reference API
    @property
    def posterior_mean(self):
        return self._pm[..., None]

    @property
    def posterior_variance(self):
        return self._pv

    def update_posterior(self):
        """Filter + smoother from the current sites (basemodels.py:689-706); also
        evaluates the site expectations and energy terms at the new posterior."""
        self._sync_params()
        _lib.check(self._lib.bn_update_posterior(self._handle, self._stream(), 1 if self.parallel else 0,
                                                 self.dt.data_ptr(), self.Y.data_ptr(), ctypes.byref(self._state)),
                   "bn_update_posterior")
        self._stale = False
        self._result = None

    def inference(self, lr=1.0, batch_ind=None, return_terms=False, **kwargs):
        """One damped natural-gradient / Newton step of the sites followed by the
        posterior update (inference.py:65-90).  With return_terms, returns
        ((mean, jacobian, hessian), (diff1, diff2)) like the reference."""
        if batch_ind is not None and batch_ind.shape[0] != self.num_data:
            raise NotImplementedError("mini-batched site updates are not supported")
        self._sync_params()
        if self._stale:
            self.update_posterior()
        terms = None
        if return_terms:
            terms = (self._lin[..., None].clone(), self._grad[..., None].clone(), self._hess.clone())
        _lib.check(self._lib.bn_newton_step(self._handle, self._stream(), 1 if self.parallel else 0, float(lr),
                                            self.dt.data_ptr(), self.Y.data_ptr(), ctypes.byref(self._state)),
                   "bn_newton_step")
        self._result = None
        if return_terms:
            res, _ = self._fetch()
            n = self.num_data * self.site_dim
            return terms, (res[_lib.RES_DIFF1] / n, res[_lib.RES_DIFF2] / (n * self.site_dim))
        return None

    def energy(self, batch_ind=None, **kwargs):
        """The energy at the current posterior: negative ELBO for VI
        (inference.py:197-222), the Laplace energy for Newton (:130-154), the EP
        energy (:286-325)."""
        self._sync_params()
        if self._stale:
            self.update_posterior()
        return self._fetch()[0][_lib.RES_ENERGY]

    def compute_log_lik(self):
        """log int p(f) N(pseudo_y | f, pseudo_var) df (basemodels.py:726-741)."""
        self._sync_params()
        if self._stale:
            self.update_posterior()
        return self._fetch()[0][_lib.RES_LOGLIK]

    def compute_kl(self):
        """KL[q || p] (basemodels.py:708-724); VI / Newton sites."""
        self._sync_params()
        if self._stale:
            self.update_posterior()
        res = self._fetch()[0]
        return res[_lib.RES_SUM2] - res[_lib.RES_LOGLIK]

    def status(self):
        """Device status bits of the last step (BN_STATUS_*)."""
        return self._fetch()[1]

    def set_profiling(self, on=True):
        """Record per-kernel CUDA events in the following steps (runs them without
        the CUDA graph)."""
        _lib.check(self._lib.bn_model_set_profiling(self._handle, 1 if on else 0), "bn_model_set_profiling")

    def kernel_times(self):
        """{kernel: ms} of the last profiled step."""
        out = (ctypes.c_float * 6)()
        _lib.check(self._lib.bn_model_kernel_times(self._handle, out, 6), "bn_model_kernel_times")
        return dict(zip(_lib.KERNELS, list(out)))

    # ------------------------------------------------------------ prediction
    def _test_times(self, X):
        X = X if isinstance(X, torch.Tensor) else torch.as_tensor(np.asarray(X))
        X = X.to(device=self.device, dtype=torch.float64)
        if X.ndim > 1:
            X = X[:, 0]  # the temporal component
        return X.contiguous()

    def predict(self, X=None, R=None):
        """Posterior mean and variance of f at test times X (default: the training
        times), basemodels.py:766-816: filter and smoother with gains from the
        current sites, then the state at each test time from its two neighbours.
        Returns ([Nt], [Nt]) for one latent, ([Nt, P], [Nt, P, P]) for P."""
        if R is not None:
            raise NotImplementedError("spatial inputs are not supported by the temporal path")
        self._sync_params()
        if self._stale:
            self.update_posterior()
        self._fetch()  # keep the last step's results and status
        xt = self._t64 if X is None else self._test_times(X)
        nt, P = xt.shape[0], self.site_dim
        mean = torch.empty(nt, P, device=self.device, dtype=self.dtype)
        cov = torch.empty(nt, P, P, device=self.device, dtype=self.dtype)
        _lib.check(self._lib.bn_model_predict(self._handle, self._stream(), 1 if self.parallel else 0,
                                              self.dt.data_ptr(), self.Y.data_ptr(), ctypes.byref(self._state),
                                              self._t64.data_ptr(), nt, xt.data_ptr(), mean.data_ptr(),
                                              cov.data_ptr()), "bn_model_predict")
        if P == 1:
            return mean[:, 0], cov[:, 0, 0]
        return mean, cov

    def predict_y(self, X=None, R=None, cubature=None):
        """Predictive mean and variance of y (basemodels.py:165-175)."""
        m, v = self.predict(X, R)
        if self.site_dim != 1:
            raise NotImplementedError("predict_y covers single-latent likelihoods")
        m, v = m.contiguous(), v.contiguous()
        my, vy = torch.empty_like(m), torch.empty_like(v)
        _lib.check(self._lib.bn_model_predict_y(self._handle, self._stream(), m.shape[0], m.data_ptr(), v.data_ptr(),
                                                my.data_ptr(), vy.data_ptr()), "bn_model_predict_y")
        return my, vy

    def negative_log_predictive_density(self, X, Y, R=None, cubature=None):
        """-nanmean_n log p(y_n | data) at the test points (basemodels.py:177-193)."""
        m, v = self.predict(X, R)
        if self.site_dim != 1:
            raise NotImplementedError("the predictive density covers single-latent likelihoods")
        y = Y if isinstance(Y, torch.Tensor) else torch.as_tensor(np.asarray(Y))
        y = y.to(device=self.device, dtype=self.dtype).reshape(-1).contiguous()
        if y.shape[0] != m.shape[0]:
            raise ValueError("Y has %d points, X %d" % (y.shape[0], m.shape[0]))
        sc = (ctypes.c_double * 2)()
        _lib.check(self._lib.bn_model_log_density(self._handle, self._stream(), y.shape[0], y.data_ptr(),
                                                  m.contiguous().data_ptr(), v.contiguous().data_ptr(), None, sc),
                   "bn_model_log_density")
        return -sc[0] / sc[1] if sc[1] > 0 else float("nan")

    # ------------------------------------------------------------ checkpoint / resume
    def state_dict(self):
        """The complete state of the iteration, host arrays: the sites (the
        reference's pseudo_likelihood state variables, basemodels.py:130-135) and the
        hyperparameters of the prior components and the likelihood."""
        out = {"nat1": self._nat1.cpu().numpy(), "nat2": self._nat2.cpu().numpy()}
        for i, c in enumerate(self.kernel.components()):
            for name in c._params:
                out["kernel.%d.%s" % (i, name)] = np.asarray(getattr(c, name), dtype=np.float64)
        for name in self.likelihood._params:
            out["likelihood.%s" % name] = np.asarray(getattr(self.likelihood, name), dtype=np.float64)
        return out

    def load_state_dict(self, state):
        """Resume from state_dict(): the sites and hyperparameters are set and the
        posterior is recomputed at the next step."""
        n1 = torch.as_tensor(np.asarray(state["nat1"]))
        n2 = torch.as_tensor(np.asarray(state["nat2"]))
        if tuple(n1.shape) != tuple(self._nat1.shape) or tuple(n2.shape) != tuple(self._nat2.shape):
            raise ValueError("site arrays do not match this model's shape")
        self._nat1.copy_(n1.to(self._nat1))
        self._nat2.copy_(n2.to(self._nat2))
        for i, c in enumerate(self.kernel.components()):
            for name in c._params:
                key = "kernel.%d.%s" % (i, name)
                if key in state:
                    v = np.asarray(state[key], dtype=np.float64)
                    setattr(c, name, float(v) if v.ndim == 0 else v)
        for name in self.likelihood._params:
            key = "likelihood.%s" % name
            if key in state:
                setattr(self.likelihood, name, float(np.asarray(state[key])))
        self._stale = True
        self._result = None

    def save(self, path):
        """state_dict() to an .npz file."""
        np.savez(path, **self.state_dict())

    def load(self, path):
        """load_state_dict() from an .npz file written by save()."""
        with np.load(path) as f:
            self.load_state_dict({k: f[k] for k in f.files})

    # ------------------------------------------------------------ hyperparameter gradient
    def hyperparameters(self):
        """[(name, object, attribute)] of the trainable hyperparameters in the order
        of energy_and_grad: 'kernel.<i>.variance', 'kernel.<i>.lengthscale' for
        every prior component, then 'likelihood.variance' for a Gaussian likelihood."""
        out = []
        for i, c in enumerate(self.kernel.components()):
            out += [("kernel.%d.variance" % i, c, "variance"), ("kernel.%d.lengthscale" % i, c, "lengthscale")]
        if self.likelihood.kind() == _lib.LIK_GAUSSIAN:
            out.append(("likelihood.variance", self.likelihood, "variance"))
        return out

    def energy_and_grad(self, transformed=False):
        """The energy of the model's method (VI, Newton, EP, PL) and its gradient with
        respect to the hyperparameters, as objax.GradValues(model.energy) gives them
        in the reference's training loop (README.md:58-66): sites and posterior
        marginals held fixed.  Returns
        (energy, {name: d energy / d value}); transformed=True differentiates with
        respect to softplus^-1(value), the reference's trainable variables."""
        energy = self.energy()
        names = self.hyperparameters()
        nc = len(self.kernel.components())
        g = (ctypes.c_double * (2 * nc + 1))()
        _lib.check(self._lib.bn_model_energy_grad(self._handle, self._stream(), 1 if self.parallel else 0,
                                                  self.dt.data_ptr(), self.Y.data_ptr(), ctypes.byref(self._state),
                                                  g, None), "bn_model_energy_grad")
        vals = list(g)[:2 * nc] + ([g[2 * nc]] if len(names) > 2 * nc else [])
        out = {}
        for (name, obj, attr), v in zip(names, vals):
            if transformed:
                v *= -math.expm1(-float(getattr(obj, attr)))  # d softplus(t) / dt = 1 - exp(-value)
            out[name] = v
        return energy, out

    # ------------------------------------------------------------ learned sites
    def site_inputs(self, augment=0, seed=0):
        """(y, m1, m2, v11, v12, v22) [n, 6] of the two-latent sites at the current
        posterior, plus `augment` jittered copies (means moved by up to a posterior
        sd, variances scaled by up to e^{+-1}) to cover the next steps' marginals."""
        if self.site_dim != 2:
            raise NotImplementedError("learned sites cover two-latent likelihoods")
        self._sync_params()
        if self._stale:
            self.update_posterior()
        pm, pv = self._pm.float(), self._pv.float()
        base = torch.stack([self.Y[:, 0].float(), pm[:, 0], pm[:, 1], pv[:, 0, 0], 0.5 * (pv[:, 0, 1] + pv[:, 1, 0]),
                            pv[:, 1, 1]], 1)
        out = [base]
        g = torch.Generator(device=base.device).manual_seed(seed)
        for _ in range(augment):
            z = torch.randn(base.shape[0], 4, device=base.device, generator=g)
            x = base.clone()
            x[:, 1] += z[:, 0] * base[:, 3].sqrt()
            x[:, 2] += z[:, 1] * base[:, 5].sqrt()
            s1, s2 = torch.exp(z[:, 2].clamp(-2, 2) * 0.5), torch.exp(z[:, 3].clamp(-2, 2) * 0.5)
            x[:, 3] = base[:, 3] * s1 * s1
            x[:, 5] = base[:, 5] * s2 * s2
            x[:, 4] = base[:, 4] * s1 * s2
            out.append(x)
        return torch.cat(out).contiguous()

    def set_surrogate(self, surrogate, spot=64, tol=0.05):
        """Site expectations from a trained CubatureSurrogate (None: cubature)."""
        h = None if surrogate is None else surrogate._h
        _lib.check(self._lib.bn_model_set_surrogate(self._handle, h, int(spot), float(tol)), "bn_model_set_surrogate")
        self._surrogate = surrogate
        self._stale = True

    def surrogate_counts(self):
        """(sites reverted for -H not PD, spot-checked sites reverted) of the last step."""
        res = self._fetch()[0]
        return int(res[_lib.RES_SURR_PSD]), int(res[_lib.RES_SURR_SPOT])

    def chunking(self):
        sd, pd, spt, nb = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._lib.bn_model_info(self._handle, ctypes.byref(sd), ctypes.byref(pd), ctypes.byref(spt), ctypes.byref(nb))
        return spt.value, nb.value


MarkovGP = MarkovGaussianProcess


class MarkovVariationalGP(MarkovGaussianProcess):
    """VI + Markov GP (models.py:118-132)."""
    _method = _lib.METHOD_VI


class MarkovNewtonGP(MarkovGaussianProcess):
    """Newton / Laplace + Markov GP (models.py:297-299)."""
    _method = _lib.METHOD_NEWTON


MarkovLaplaceGP = MarkovNewtonGP


class MarkovExpectationPropagationGP(MarkovGaussianProcess):
    """Power EP + Markov GP (models.py:216-231)."""
    _method = _lib.METHOD_EP

    def __init__(self, kernel, likelihood, X, Y, R=None, power=1.0, parallel=None, **kw):
        super().__init__(kernel, likelihood, X, Y, R=R, parallel=parallel, power=power, **kw)


MarkovEPGP = MarkovExpectationPropagationGP


class MarkovPosteriorLinearisationGP(MarkovGaussianProcess):
    """Posterior linearisation + Markov GP (models.py:361-377, inference.py:328-428):
    sites from the statistical linear regression of the likelihood at the posterior
    marginals (no positive-precision fix: -dmu^2 / omega is never positive), energy
    the EP energy at power 1.  Single-latent likelihoods."""
    _method = _lib.METHOD_PL

    def __init__(self, kernel, likelihood, X, Y, R=None, parallel=None, **kw):
        kw.pop("power", None)
        super().__init__(kernel, likelihood, X, Y, R=R, parallel=parallel, power=1.0, **kw)

    def _lik_desc(self):
        return self.likelihood.desc(self._method, self.cubature.num_cub_points, 1.0, False, self.score_form)


MarkovPLGP = MarkovPosteriorLinearisationGP


def _mean_field_kernel(kernel):
    if not isinstance(kernel, Independent) or isinstance(kernel, Sum):
        raise ValueError("the mean-field models take an Independent prior (one block per latent)")


class MarkovVariationalMeanFieldGP(MarkovVariationalGP):
    """VI + the mean-field Markov GP (models.py:154-155, basemodels.py:1158-1175),
    whose filter and smoother keep the latents' covariance block-diagonal
    (ops.py:429-706).  The VI site update keeps the site precisions diagonal
    (ensure_diagonal_positive_precision, utils.py:89-96), so with an Independent
    prior the joint filter's covariance is block-diagonal already: the joint scan
    computes the mean-field posterior exactly."""

    def __init__(self, kernel, likelihood, X, Y, R=None, **kw):
        _mean_field_kernel(kernel)
        super().__init__(kernel, likelihood, X, Y, R=R, **kw)


class MarkovNewtonMeanFieldGP(MarkovNewtonGP):
    """Newton + the mean-field Markov GP (models.py:307-308); diagonal site
    precisions as in MarkovVariationalMeanFieldGP, so the joint scan is exact."""

    def __init__(self, kernel, likelihood, X, Y, R=None, **kw):
        _mean_field_kernel(kernel)
        super().__init__(kernel, likelihood, X, Y, R=R, **kw)
