"""Oracle models: Markov GP (VI / Newton / EP) and the dense VI GP.

Follows bayesnewton/basemodels.py (GaussianDistribution :52-100, BaseModel
:103-262 with predict_y / negative_log_predictive_density :165-193, GaussianProcess
:265-378, MarkovGaussianProcess :625-816 with predict :766-816) and
bayesnewton/inference.py (newton_update :21-39, InferenceMixin.inference :65-90,
Newton :99-154, VariationalInference :160-222, ExpectationPropagation :225-325,
PosteriorLinearisation :328-428),
with utils.py input_admin (:234-265), ensure_diagonal_positive_precision
(:89-96), gaussian_expected_log_lik (:510-531) and compute_cavity (:534-541).
"""
import math

import numpy as np

from . import ops
from .kernels import Independent
from .likelihoods import pep_constant

LOG2PI = math.log(2 * math.pi)
INV2PI = (2 * math.pi) ** -1


def input_admin(t, y):
    """Sort by time; dt = [0, diff(t)] (utils.py:234-265, temporal case)."""
    t = np.asarray(t, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    if t.ndim < 2:
        t = t[:, None]
    if y.ndim < 2:
        y = y[:, None]
    ind = np.argsort(t[:, 0], axis=0, kind="stable")
    t, y = t[ind], y[ind]
    dt = np.concatenate([[0.0], np.diff(t[:, 0])])
    return t, y, dt


def ensure_diagonal_positive_precision(K):
    """Keep diag(K), replace negatives with 1e-2, drop off-diagonals (utils.py:89-96)."""
    d = np.diagonal(K, axis1=-2, axis2=-1)
    d = np.where(d < 0, 1e-2, d)
    return d[..., :, None] * np.eye(K.shape[-1])


def newton_update(mean, jacobian, hessian):
    """Natural-parameter Newton step with the NaN (missing data) rule (inference.py:21-39)."""
    hessian = np.where(np.isnan(hessian), -1e-6, hessian)
    jacobian = np.where(np.isnan(jacobian), hessian @ mean, jacobian)
    return jacobian - hessian @ mean, -hessian


def gaussian_expected_log_lik(Y, q_mu, q_covar, noise, mask=None):
    """E_q log N(Y | f, noise), q = N(q_mu, q_covar), masked (utils.py:510-531)."""
    Y = Y.reshape(-1, 1)
    q_mu = q_mu.reshape(-1, 1)
    q_covar = np.array(q_covar, dtype=np.float64)
    noise = np.array(noise, dtype=np.float64)
    if mask is not None:
        maskv = np.asarray(mask, dtype=bool).reshape(-1, 1)
        q_mu = np.where(maskv, Y, q_mu)
        noise = np.where(maskv | maskv.T, 0.0, noise)
        noise = np.where(np.diag(maskv[:, 0]), INV2PI, noise)
        q_covar = np.where(maskv | maskv.T, 0.0, q_covar)
        q_covar = np.where(np.diag(maskv[:, 0]), 1e-20, q_covar)
    ml = ops.mvn_logpdf(Y, q_mu, noise)
    return ml - 0.5 * np.trace(ops.solve(noise, q_covar))


def reparametrise(p1, p2):
    """(mean, cov) <-> (nat1, nat2) via per-site Cholesky (basemodels.py:85-90)."""
    return ops.solve(p2, p1), ops.inv(p2)


def compute_cavity(post_mean, post_cov, site_nat1, site_nat2, power, jitter=1e-8):
    """utils.py:534-541."""
    post_nat2 = ops.inv(post_cov + jitter * np.eye(post_cov.shape[1]))
    cav_cov = ops.inv(post_nat2 - power * site_nat2)
    cav_mean = cav_cov @ (post_nat2 @ post_mean - power * site_nat1)
    return cav_mean, cav_cov


class _Base:
    """Sites and posterior containers shared by the dense and Markov models
    (basemodels.py:103-144)."""

    def _init_common(self, kernel, likelihood, X, Y, func_dim):
        self.kernel = kernel
        self.likelihood = likelihood
        self.X, self.Y = X, Y
        self.num_data = X.shape[0]
        self.func_dim = func_dim
        self.obs_dim = Y.shape[1]
        p = func_dim if isinstance(kernel, Independent) else self.obs_dim
        self.site_dim = p
        self.site_mean = np.zeros([self.num_data, p, 1])
        self.site_cov = 1e2 * np.tile(np.eye(p), [self.num_data, 1, 1])
        self.site_nat1, self.site_nat2 = reparametrise(self.site_mean, self.site_cov)
        self.posterior_mean = np.zeros([self.num_data, func_dim, 1])
        self.posterior_variance = np.tile(np.eye(func_dim), [self.num_data, 1, 1])
        self.mask_y = np.isnan(Y).reshape(Y.shape[0], Y.shape[1])
        if func_dim == self.obs_dim:
            self.mask_pseudo_y = self.mask_y
        elif likelihood.multi_latent:
            self.mask_pseudo_y = None
        else:
            self.mask_pseudo_y = np.tile(self.mask_y, [1, p])

    def update_nat_params(self, nat1, nat2):
        self.site_nat1, self.site_nat2 = nat1, nat2
        self.site_mean, self.site_cov = reparametrise(nat1, nat2)

    def predict_y(self, X_test):
        """basemodels.py:165-175 for a single-latent likelihood."""
        m, v = self.predict(X_test)
        out = np.array([self.likelihood.predict(mi, vi) for mi, vi in zip(np.atleast_1d(m), np.atleast_1d(v))])
        return out[:, 0], out[:, 1]

    def negative_log_predictive_density(self, X_test, Y_test):
        """basemodels.py:177-193 for a single-latent likelihood: -nanmean of the
        log predictive density, NaN observations left out."""
        m, v = self.predict(X_test)
        y = np.asarray(Y_test, dtype=np.float64).reshape(-1)
        ld = np.array([np.nan if np.isnan(yi) else self.likelihood.log_density(yi, mi, vi)
                       for yi, mi, vi in zip(y, np.atleast_1d(m), np.atleast_1d(v))])
        return float(-np.nanmean(ld))

    def expected_density_pseudo(self, pseudo_y=None, pseudo_var=None):
        if pseudo_y is None:
            pseudo_y, pseudo_var = self.site_mean, self.site_cov
        tot = 0.0
        for n in range(self.num_data):
            tot += gaussian_expected_log_lik(
                pseudo_y[n], self.posterior_mean[n], self.posterior_variance[n], pseudo_var[n],
                None if self.mask_pseudo_y is None else self.mask_pseudo_y[n])
        return tot

    # ---------------------------------------------------------------- site updates
    def _site_expectations(self, mean_f, cov_f):
        lik = self.likelihood
        ell = np.zeros(self.num_data)
        d1 = np.zeros([self.num_data, self.site_dim, 1])
        d2 = np.zeros([self.num_data, self.site_dim, self.site_dim])
        for n in range(self.num_data):
            e, g, h = lik.variational_expectation(self.Y[n], mean_f[n], cov_f[n])
            ell[n], d1[n], d2[n] = e, np.reshape(g, (-1, 1)), h
        return ell, d1, d2

    def _newton_derivs(self, mean_f):
        lik = self.likelihood
        ll = np.zeros(self.num_data)
        d1 = np.zeros([self.num_data, self.site_dim, 1])
        d2 = np.zeros([self.num_data, self.site_dim, self.site_dim])
        for n in range(self.num_data):
            l, g, h = lik.log_likelihood_gradients(self.Y[n], mean_f[n])
            ll[n], d1[n], d2[n] = l, np.reshape(g, (-1, 1)), np.reshape(h, (self.site_dim, self.site_dim))
        return ll, d1, d2

    def update_variational_params(self, method="vi", ensure_psd=True, power=1.0):
        """VI (inference.py:170-195), Newton (:105-128) or EP (:238-284)."""
        if method == "vi":
            mean_f, cov_f = self.posterior_mean, self.posterior_variance
            _, jac, hess = self._site_expectations(mean_f, cov_f)
            if ensure_psd:
                hess = -ensure_diagonal_positive_precision(-hess)
            return mean_f, jac, hess
        if method == "newton":
            mean_f = self.posterior_mean
            _, jac, hess = self._newton_derivs(mean_f)
            if ensure_psd:
                hess = -ensure_diagonal_positive_precision(-hess)
            return mean_f, jac, hess
        if method == "ep":
            cav_mean, cav_cov = compute_cavity(self.posterior_mean, self.posterior_variance,
                                               self.site_nat1, self.site_nat2, power)
            lik = self.likelihood
            dl = np.zeros([self.num_data, self.site_dim, 1])
            d2l = np.zeros([self.num_data, self.site_dim, self.site_dim])
            for n in range(self.num_data):
                _, a, b = lik.moment_match(self.Y[n], cav_mean[n], cav_cov[n], power)
                dl[n], d2l[n] = a, b
            cav_prec = ops.inv(cav_cov)
            scale = cav_prec @ ops.inv(d2l + cav_prec) / power
            dl = scale @ dl
            d2l = scale @ d2l
            if self.mask_pseudo_y is not None:
                mask = self.mask_pseudo_y[..., None]
                dl = np.where(mask, np.nan, dl)
                d2l_m = np.where(mask | np.swapaxes(mask, -1, -2), 0.0, d2l)
                diagm = mask[..., 0][..., :, None] * np.eye(self.site_dim, dtype=bool)
                d2l = np.where(diagm, np.nan, d2l_m)
            if ensure_psd:
                hess = -ensure_diagonal_positive_precision(-d2l)
            else:
                hess = d2l
            return cav_mean, dl, hess
        if method == "pl":
            # PosteriorLinearisation.update_variational_params (inference.py:339-369),
            # single-latent sites; no positive-precision fix
            mean_f, cov_f = self.posterior_mean, self.posterior_variance
            jac = np.zeros([self.num_data, 1, 1])
            hess = np.zeros([self.num_data, 1, 1])
            for n in range(self.num_data):
                mu, omega, dmu = self.likelihood.statistical_linear_regression(mean_f[n, 0, 0], cov_f[n, 0, 0])
                y = self.Y[n, 0]
                if np.isnan(y):
                    res, omega = 0.0, 1e6
                else:
                    res = y - mu
                jac[n, 0, 0] = dmu / omega * res
                hess[n, 0, 0] = -dmu / omega * dmu
            return mean_f, jac, hess
        raise ValueError(method)

    def inference(self, lr=1.0, method="vi", power=1.0, ensure_psd=True):
        """InferenceMixin.inference (inference.py:65-90)."""
        self.update_posterior()
        mean, jac, hess = self.update_variational_params(method, ensure_psd, power)
        nat1_n, nat2_n = newton_update(mean, jac, hess)
        diff1 = np.mean(np.abs(nat1_n - self.site_nat1))
        diff2 = np.mean(np.abs(nat2_n - self.site_nat2))
        self.update_nat_params((1 - lr) * self.site_nat1 + lr * nat1_n,
                               (1 - lr) * self.site_nat2 + lr * nat2_n)
        self.update_posterior()
        return (mean, jac, hess), (diff1, diff2)

    # ---------------------------------------------------------------- energies
    def energy(self, method="vi", power=1.0):
        if method == "vi":
            ell, _, _ = self._site_expectations(self.posterior_mean, self.posterior_variance)
            return -(np.nansum(ell) - self.compute_kl())
        if method == "newton":
            ll, _, _ = self._newton_derivs(self.posterior_mean)
            return -(np.nansum(ll) - self.compute_kl())
        if method == "ep":
            return self.ep_energy(power)
        if method == "pl":
            # PosteriorLinearisation.energy (inference.py:371-428): the EP energy at power 1
            return self.ep_energy(1.0)
        raise ValueError(method)

    def compute_kl(self):
        """KL[q||p] = sum E_q log N(pseudo_y | f, pseudo_var) - log Z_pseudo
        (basemodels.py:708-724 and :355-364)."""
        return self.expected_density_pseudo() - self.compute_log_lik()

    def ep_energy(self, power):
        """ExpectationPropagation.energy (inference.py:286-325) with
        compute_ep_energy_terms (basemodels.py:241-262), single-latent sites."""
        cav_mean, cav_cov = compute_cavity(self.posterior_mean, self.posterior_variance,
                                           self.site_nat1, self.site_nat2, power)
        lel_pseudo = 0.0
        for n in range(self.num_data):
            m = None if self.mask_pseudo_y is None else self.mask_pseudo_y[n]
            lel_pseudo += ops.mvn_logpdf(self.site_mean[n], cav_mean[n],
                                         self.site_cov[n] / power + cav_cov[n], m)
            if m is None or not np.any(m):
                lel_pseudo += pep_constant(self.site_cov[n], power)
            else:
                # pep_constant with mask (utils.py:431-446)
                L = np.linalg.cholesky(self.site_cov[n])
                ldc = np.where(m, 0.0, np.log(np.abs(np.diag(L))))
                dim = self.site_cov[n].shape[1] - int(np.sum(m))
                lel_pseudo += 0.5 * dim * ((1 - power) * LOG2PI - np.log(power)) \
                    + 0.5 * (1 - power) * 2 * np.sum(ldc)
        lZ = self.compute_log_lik()
        lel = np.zeros(self.num_data)
        for n in range(self.num_data):
            lel[n] = self.likelihood.moment_match(self.Y[n], cav_mean[n], cav_cov[n], power)[0]
        lel = np.where(np.squeeze(self.mask_y), 0.0, lel)
        return -(lZ + 1.0 / power * (np.nansum(lel) - lel_pseudo))


class MarkovGP(_Base):
    """MarkovGaussianProcess, temporal case (basemodels.py:625-764)."""

    def __init__(self, kernel, likelihood, X, Y, parallel=False, stable=False):
        X, Y, self.dt = input_admin(X, Y)
        H = kernel.measurement_model()
        self._init_common(kernel, likelihood, X, Y, func_dim=H.shape[0])
        self.parallel = parallel
        # stable: the parallel filter combines with (I + C1 J2)^-1 instead of the
        # reference's inv(C1), which fails when C1 is singular to working precision
        self.stable = stable
        self.last_log_lik = None

    def update_posterior(self):
        """basemodels.py:689-706 (the smoother uses dt shifted by one)."""
        ell, (fm, fP) = ops.kalman_filter(self.dt, self.kernel, self.site_mean, self.site_cov,
                                          mask=self.mask_pseudo_y, parallel=self.parallel,
                                          stable=self.stable)
        self.last_log_lik = ell
        dts = np.concatenate([self.dt[1:], [0.0]])
        sm, sP, _ = ops.rauch_tung_striebel_smoother(dts, self.kernel, fm, fP,
                                                     parallel=self.parallel)
        self.posterior_mean, self.posterior_variance = sm, sP

    def compute_log_lik(self):
        """basemodels.py:726-741."""
        ell, _ = ops.kalman_filter(self.dt, self.kernel, self.site_mean, self.site_cov,
                                   mask=self.mask_pseudo_y, parallel=self.parallel, stable=self.stable)
        return ell

    def predict(self, X_test):
        """basemodels.py:766-816, temporal case: filter, full smoother with gains,
        then the state at each test time from its two neighbours."""
        _, (fm, fP) = ops.kalman_filter(self.dt, self.kernel, self.site_mean, self.site_cov,
                                        mask=self.mask_pseudo_y, parallel=self.parallel)
        dts = np.concatenate([self.dt[1:], [0.0]])
        sm, sP, G = ops.rauch_tung_striebel_smoother(dts, self.kernel, fm, fP, return_full=True,
                                                     parallel=self.parallel)
        X_aug = np.concatenate([[-1e10], self.X[:, 0], [1e10]])
        m, P = ops.temporal_conditional(X_aug, X_test, sm, sP, G, self.kernel)
        H = self.kernel.measurement_model()
        return np.squeeze(H @ m), np.squeeze(H @ P @ H.T)


class MarkovMeanFieldGP(MarkovGP):
    """MarkovMeanFieldGaussianProcess (basemodels.py:1158-1175): an Independent prior
    whose filter and smoother keep the latents' covariance block-diagonal
    (ops.py:429-706), sequential form."""

    def __init__(self, kernel, likelihood, X, Y, parallel=False):
        super().__init__(kernel, likelihood, X, Y, parallel=parallel)
        self.block_sizes = [k.state_dim for k in kernel.kernels]

    def update_posterior(self):
        ell, (fm, fP) = ops.kalman_filter_meanfield(self.dt, self.kernel, self.site_mean, self.site_cov,
                                                    mask=self.mask_pseudo_y, block_sizes=self.block_sizes)
        self.last_log_lik = ell
        dts = np.concatenate([self.dt[1:], [0.0]])
        self.posterior_mean, self.posterior_variance = ops.rauch_tung_striebel_smoother_meanfield(
            dts, self.kernel, fm, fP, block_sizes=self.block_sizes)

    def compute_log_lik(self):
        return ops.kalman_filter_meanfield(self.dt, self.kernel, self.site_mean, self.site_cov,
                                           mask=self.mask_pseudo_y, block_sizes=self.block_sizes)[0]


class InfiniteHorizonGP(MarkovGP):
    """InfiniteHorizonGaussianProcess (basemodels.py:1257-1308), temporal case:
    equidistant times, the filter and smoother hooks replaced by their
    infinite-horizon forms, the Riccati recursions warm-started from the previous
    call's solutions (state variables there, Pinf at first)."""

    def __init__(self, kernel, likelihood, X, Y, dare_iters=20, parallel=False):
        super().__init__(kernel, likelihood, X, Y, parallel=parallel)
        if self.dt.shape[0] > 2 and np.max(np.abs(np.diff(self.dt[1:]))) >= 1e-6:
            raise ValueError("time steps must be equidistant")
        self.heteroscedastic = bool(np.any(np.isnan(self.Y))) or likelihood.name != "gaussian"
        self.dare_iters = dare_iters
        Pinf = kernel.stationary_covariance()
        self.dare_init_filter = Pinf
        self.dare_init_smoother = Pinf

    def _filter(self):
        tied = np.mean(self.site_nat2, axis=0)
        out = ops.kalman_filter_infinite_horizon(
            self.dt, self.kernel, self.site_mean, self.site_cov, mask=self.mask_pseudo_y, parallel=self.parallel,
            heteroscedastic=self.heteroscedastic, noise_cov_tied=np.linalg.inv(tied), dare_iters=self.dare_iters,
            dare_init=self.dare_init_filter)
        self.dare_init_filter = out[1][1][0]
        return out

    def update_posterior(self):
        ell, (fm, fcov) = self._filter()
        self.last_log_lik = ell
        dts = np.concatenate([self.dt[1:], [0.0]])
        sm, sP, _, dcov = ops.rauch_tung_striebel_smoother_infinite_horizon(
            dts, self.kernel, fm, fcov, parallel=self.parallel, dare_iters=self.dare_iters,
            dare_init=self.dare_init_smoother)
        self.dare_init_smoother = dcov
        self.posterior_mean, self.posterior_variance = sm, sP

    def compute_log_lik(self):
        return self._filter()[0]


class DenseGP(_Base):
    """GaussianProcess (basemodels.py:265-378) with ops.gaussian_conditional (ops.py:52-80)."""

    def __init__(self, kernel, likelihood, X, Y):
        X = np.asarray(X, dtype=np.float64)
        Y = np.asarray(Y, dtype=np.float64)
        if X.ndim < 2:
            X = X[:, None]
        if Y.ndim < 2:
            Y = Y[:, None]
        # the reference counts latents with isinstance(kernel, Independent), which also
        # matches Sum (a subclass); the dense model is only a test oracle here, so a
        # Sum prior is treated as the single latent it is
        fd = kernel.num_kernels if type(kernel) is Independent else 1
        self._init_common(kernel, likelihood, X, Y, func_dim=fd)

    def _noise_block(self, cov):
        N, p = cov.shape[0], cov.shape[1]
        B = np.zeros([N * p, N * p])
        for n in range(N):
            B[n * p:(n + 1) * p, n * p:(n + 1) * p] = cov[n]
        return B

    def update_posterior(self):
        Kff = self.kernel(self.X, self.X)
        Ky = Kff + self._noise_block(self.site_cov)
        KiKy = ops.solve(Ky, Kff).T
        mean = KiKy @ self.site_mean.reshape(-1, 1)
        cov = Kff - KiKy @ Kff
        p = self.func_dim
        self.posterior_mean = mean.reshape(self.num_data, p, 1)
        self.posterior_variance = np.stack(
            [cov[n * p:(n + 1) * p, n * p:(n + 1) * p] for n in range(self.num_data)])

    def predict(self, X_test):
        """GaussianProcess.predict (basemodels.py:331-345) through
        ops.gaussian_conditional (ops.py:52-80) at the test inputs."""
        Xs = np.asarray(X_test, dtype=np.float64)
        if Xs.ndim < 2:
            Xs = Xs[:, None]
        Kff = self.kernel(self.X, self.X)
        Kfs = self.kernel(self.X, Xs)
        Kss = self.kernel(Xs, Xs)
        Ky = Kff + self._noise_block(self.site_cov)
        Kfs_iKy = ops.solve(Ky, Kfs).T
        mean = Kfs_iKy @ self.site_mean.reshape(-1, 1)
        cov = Kss - Kfs_iKy @ Kfs
        p = self.func_dim
        n = Xs.shape[0]
        var = np.stack([cov[i * p:(i + 1) * p, i * p:(i + 1) * p] for i in range(n)])
        return np.squeeze(mean.reshape(n, p)), np.squeeze(var)

    def compute_log_lik(self):
        Ky = self.kernel(self.X, self.X) + self._noise_block(self.site_cov)
        y = self.site_mean.reshape(-1, 1)
        L = np.linalg.cholesky(Ky)
        z = np.linalg.solve(L, y)
        return float(-0.5 * (z.T @ z).item() - np.sum(np.log(np.diag(L))) - 0.5 * y.shape[0] * LOG2PI)


def hyperparameters(model):
    """(object, attribute) pairs of the trainable hyperparameters in the order the
    library reports their gradient: variance then lengthscale of every prior
    component, then a Gaussian likelihood's noise variance."""
    k = model.kernel
    comps = k.kernels if hasattr(k, "kernels") else [k]
    out = []
    for c in comps:
        out += [(c, "variance"), (c, "lengthscale")]
    if hasattr(model.likelihood, "variance") and model.likelihood.name == "gaussian":
        out.append((model.likelihood, "variance"))
    return out


def energy_gradient_fd(model, rel_step=1e-5, method="vi", power=1.0):
    """d energy / d theta as objax.GradValues(model.energy) gives it (README.md:58-66):
    the sites and the stored posterior (state variables in the reference) held
    fixed, the energy re-evaluated at perturbed hyperparameters.  Central
    differences with step rel_step * theta (error ~ rel_step^2 relative)."""
    grads = []
    for obj, name in hyperparameters(model):
        v0 = getattr(obj, name)
        h = rel_step * v0
        setattr(obj, name, v0 + h)
        ep = model.energy(method, power)
        setattr(obj, name, v0 - h)
        em = model.energy(method, power)
        setattr(obj, name, v0)
        grads.append((ep - em) / (2.0 * h))
    return np.array(grads)

