"""Oracle likelihoods (float64 numpy restatement).

Per-site routines take scalars (single-latent) or small arrays (multi-latent) and
follow bayesnewton/likelihoods.py:
  - Likelihood.variational_expectation masking (:363-383), moment_match (:401-412),
    log_likelihood_gradients (:326-355);
  - Gaussian (:684-803): closed-form VE and moment matching;
  - Bernoulli (:806-860): logit or probit (jitter 1e-3) link, VE by 20-point GH;
  - Poisson (:891-1008): exp link, closed-form VE;
  - log_density (:385-388 -> cubature.py:249-276; Gaussian closed form :784-800) and
    predict (:493-506 -> cubature.py:438-465 with conditional_moments; Gaussian
    :802-803) for single-latent likelihoods;
  - HeteroscedasticNoise (:1244-1281) with MultiLatentLikelihood.variational_expectation
    (:613-664): 2-D GH over the two latents.  The reference differentiates the
    cubature sum with autodiff; the sum's mean derivatives equal the weighted sums
    of the per-point gradient / Hessian of log p, which are written out here.
"""
import math

import numpy as np
from scipy.special import gammaln, ndtr

from .cubature import gauss_hermite, moment_match_cubature, variational_expectation_cubature

LOG2PI = math.log(2 * math.pi)
INV2PI = (2 * math.pi) ** -1


def mvn_logpdf_and_derivs(x, mean, cov):
    """utils.py:448-466 without a mask."""
    n = mean.shape[0]
    L = np.linalg.cholesky(cov)
    prec = np.linalg.inv(cov)
    log_det = 2 * np.sum(np.log(np.abs(np.diag(L))))
    diff = x - mean
    sd = prec @ diff
    dist = (diff.T @ sd).item()
    return -0.5 * (dist + n * LOG2PI + log_det), sd, -prec


def pep_constant(var, power):
    """utils.py:431-446 without a mask."""
    dim = var.shape[1]
    L = np.linalg.cholesky(var)
    logdet = 2 * np.sum(np.log(np.abs(np.diag(L))))
    return 0.5 * dim * ((1 - power) * LOG2PI - np.log(power)) + 0.5 * (1 - power) * logdet


class Likelihood:
    multi_latent = False
    num_cub = 20

    # --- per-site VE for one scalar output (likelihoods.py:357-361) ---
    def ve_scalar(self, y, m, v):
        return variational_expectation_cubature(self.log_lik, y, m, v, self.num_cub)

    def variational_expectation(self, y, m, v):
        """y [p,1] (NaN = missing), m [p,1], v [p,p] -> (E scalar, dE [p,1], d2E [p,p])
        following likelihoods.py:363-383 (per output dim, NaN mask)."""
        y = np.asarray(y, dtype=np.float64).reshape(-1)
        m = np.asarray(m, dtype=np.float64).reshape(-1)
        v = np.diag(np.atleast_2d(v)).reshape(-1)
        mask = np.isnan(y)
        y = np.where(mask, m, y)
        E = np.zeros(y.shape[0])
        dE = np.zeros(y.shape[0])
        d2E = np.zeros(y.shape[0])
        for i in range(y.shape[0]):
            E[i], dE[i], d2E[i] = self.ve_scalar(y[i], m[i], v[i])
        E = np.where(mask, 0.0, E)
        dE = np.where(mask, np.nan, dE)
        d2E = np.where(mask, np.nan, d2E)
        return np.sum(E), dE[:, None], np.diag(d2E)

    # --- point derivatives for Newton / Laplace (likelihoods.py:326-355) ---
    def log_likelihood_gradients(self, y, f):
        y = np.asarray(y, dtype=np.float64).reshape(-1)
        f = np.asarray(f, dtype=np.float64).reshape(-1)
        mask = np.isnan(y)
        y = np.where(mask, f, y)
        ll = np.array([self.log_lik(y[i], f[i]) for i in range(y.shape[0])], dtype=np.float64)
        J = np.array([self.dlog_lik(y[i], f[i]) for i in range(y.shape[0])])
        H = np.array([self.d2log_lik(y[i], f[i]) for i in range(y.shape[0])])
        ll = np.where(mask, 0.0, ll)
        J = np.where(mask, np.nan, J)
        H = np.where(mask, np.nan, H)
        return (ll[0] if ll.shape[0] == 1 else ll), J, np.diag(H)

    # --- EP moment matching (likelihoods.py:401-412, cubature.py:310-371) ---
    def moment_match(self, y, m, v, power=1.0):
        y = np.asarray(y, dtype=np.float64).reshape(-1, 1)
        m = np.asarray(m, dtype=np.float64).reshape(-1, 1)
        mask = np.isnan(y)
        y = np.where(mask, m, y)
        return self.moment_match_(y, m, np.atleast_2d(v), power)

    def moment_match_(self, y, m, v, power):
        def ll(yy, f):
            return self.log_lik(yy[0, 0], f[0])
        return moment_match_cubature(ll, y, m, v, power, self.num_cub)

    # --- predictive densities (likelihoods.py:385-388, 493-506) ---
    def log_density(self, y, m, v):
        """log sum_i w_i p(y | sqrt(v) x_i + m), the sum floored at 1e-8
        (cubature.py:249-276)."""
        x, w = gauss_hermite(1, self.num_cub)
        f = np.sqrt(v) * x[0] + m
        Z = np.sum(w * np.exp(self.log_lik(y, f)))
        return float(np.log(max(Z, 1e-8)))

    def statistical_linear_regression(self, m, v):
        """(mu, omega, dmu/dm) of one scalar site at N(m, v) by cubature
        (cubature.py:374-430): mu = sum_i w_i E[y|f_i], omega = S - C^2 / v with
        S = sum_i w_i ((E[y|f_i] - mu)^2 + Var[y|f_i]) and C = sum_i w_i (f_i - m)
        (E[y|f_i] - mu); dmu/dm (jacrev there) = sum_i w_i dE[y|f]/df at f_i, the
        nodes f_i = sqrt(v) x_i + m moving with m."""
        x, w = gauss_hermite(1, self.num_cub)
        f = np.sqrt(v) * x[0] + m
        ey, vy = self.conditional_moments(f)
        mu = np.sum(w * ey)
        S = np.sum(w * ((ey - mu) ** 2 + vy))
        C = np.sum(w * (f - m) * (ey - mu))
        return float(mu), float(S - C * C / v), float(np.sum(w * self.d_conditional_mean(f)))

    def predict(self, m, v):
        """Data-space mean and variance by cubature of the conditional moments
        (cubature.py:438-465)."""
        x, w = gauss_hermite(1, self.num_cub)
        f = np.sqrt(v) * x[0] + m
        ey, vy = self.conditional_moments(f)
        mean = np.sum(w * ey)
        return float(mean), float(np.sum(w * (vy + ey * ey)) - mean * mean)


class Gaussian(Likelihood):
    name = "gaussian"

    def __init__(self, variance=0.1):
        self.variance = float(variance)

    def log_lik(self, y, f):
        return -0.5 * np.log(2 * np.pi * self.variance) - 0.5 * (y - f) ** 2 / self.variance

    def dlog_lik(self, y, f):
        return (y - f) / self.variance

    def d2log_lik(self, y, f):
        return -1.0 / self.variance + 0.0 * f

    def ve_scalar(self, y, m, v):
        # likelihoods.py:727-753
        E = -0.5 * np.log(2 * np.pi) - 0.5 * np.log(self.variance) - 0.5 * ((y - m) ** 2 + v) / self.variance
        return E, (y - m) / self.variance, -1.0 / self.variance

    def conditional_moments(self, f):
        return f, self.variance + 0.0 * f           # likelihoods.py:719-725

    def d_conditional_mean(self, f):
        return 1.0 + 0.0 * f

    def log_density(self, y, m, v):
        # likelihoods.py:784-800: log N(y | m, sigma^2 + v)
        s = self.variance + v
        return float(-0.5 * (LOG2PI + np.log(s) + (y - m) ** 2 / s))

    def predict(self, m, v):
        return float(m), float(v + self.variance)  # likelihoods.py:802-803

    def moment_match_(self, y, m, v, power):
        # likelihoods.py:755-780
        lik_cov = self.variance * np.eye(v.shape[0])
        lZ, dlZ, d2lZ = mvn_logpdf_and_derivs(y, m, lik_cov / power + v)
        return lZ + pep_constant(lik_cov, power), dlZ, d2lZ


class Bernoulli(Likelihood):
    name = "bernoulli"

    def __init__(self, link="probit"):
        if link not in ("probit", "logit"):
            raise NotImplementedError("link function not implemented")
        self.link = link
        self.jitter = 1e-3

    def link_fn(self, f):
        if self.link == "logit":
            return 1.0 / (1.0 + np.exp(-f))        # likelihoods.py:822
        j = self.jitter                            # likelihoods.py:826-827
        return ndtr(f) * (1 - 2 * j) + j

    def log_lik(self, y, f):
        p = self.link_fn(f)
        return np.log(np.where(np.equal(y, 1), p, 1 - p))

    def conditional_moments(self, f):
        p = self.link_fn(f)                       # likelihoods.py:854-860
        return p, p - p * p

    def d_conditional_mean(self, f):
        return self._dlink(f)[0]

    def _dlink(self, f):
        if self.link == "logit":
            s = 1.0 / (1.0 + np.exp(-f))
            return s * (1 - s), s * (1 - s) * (1 - 2 * s)
        j = self.jitter
        phi = np.exp(-0.5 * f * f) / np.sqrt(2 * np.pi)
        return phi * (1 - 2 * j), -f * phi * (1 - 2 * j)

    def dlog_lik(self, y, f):
        p = self.link_fn(f)
        d1, _ = self._dlink(f)
        return np.where(np.equal(y, 1), d1 / p, -d1 / (1 - p))

    def d2log_lik(self, y, f):
        p = self.link_fn(f)
        d1, d2 = self._dlink(f)
        return np.where(np.equal(y, 1), d2 / p - (d1 / p) ** 2, -d2 / (1 - p) - (d1 / (1 - p)) ** 2)


class Poisson(Likelihood):
    name = "poisson"

    def __init__(self, binsize=1.0, link="exp"):
        if link != "exp":
            raise NotImplementedError("only the exp link is restated")
        self.binsize = float(binsize)

    def log_lik(self, y, f):
        mu = np.exp(f) * self.binsize
        return y * np.log(mu) - mu - gammaln(y + 1)

    def dlog_lik(self, y, f):
        return y - np.exp(f) * self.binsize

    def conditional_moments(self, f):
        mu = np.exp(f) * self.binsize             # likelihoods.py:952-959
        return mu, mu

    def d_conditional_mean(self, f):
        return np.exp(f) * self.binsize

    def d2log_lik(self, y, f):
        return -np.exp(f) * self.binsize

    def ve_scalar(self, y, m, v):
        # likelihoods.py:979-1008
        emc = self.binsize * np.exp(m + v / 2)
        E = y * np.log(self.binsize) + y * m - emc - gammaln(y + 1.0)
        return E, y - emc, -emc


class HeteroscedasticNoise(Likelihood):
    """p(y | f1, f2) = N(y | f1, link(f2)^2) (likelihoods.py:1244-1281)."""
    name = "heteroscedastic"
    multi_latent = True

    def __init__(self, link="softplus"):
        if link not in ("exp", "softplus"):
            raise NotImplementedError("link function not implemented")
        self.link = link

    def _s(self, f2):
        """(s, ds, d2s): the link and its derivatives."""
        if self.link == "exp":
            e = np.exp(f2)
            return e, e, e
        sp = np.log(1.0 + np.exp(f2))
        sg = 1.0 / (1.0 + np.exp(-f2))
        return sp, sg, sg * (1 - sg)

    def log_lik(self, y, f):
        """f [2, Q] -> [Q]"""
        s, _, _ = self._s(f[1])
        return -0.5 * np.log(2 * np.pi * s * s) - 0.5 * (y - f[0]) ** 2 / (s * s)

    def grad_hess(self, y, f):
        """gradient [2, Q] and Hessian [2, 2, Q] of log p w.r.t. f."""
        s, ds, d2s = self._s(f[1])
        r = y - f[0]
        is2 = 1.0 / (s * s)
        g1 = r * is2
        g2 = -ds / s + r * r * ds / (s ** 3)
        h11 = -is2
        h12 = -2.0 * r * ds / (s ** 3)
        h22 = -(d2s * s - ds * ds) / (s * s) + r * r * (d2s / s ** 3 - 3.0 * ds * ds / s ** 4)
        return np.stack([g1, g2]), np.array([[h11, h12], [h12, h22]])

    def variational_expectation(self, y, m, v):
        """MultiLatentLikelihood.variational_expectation (likelihoods.py:613-664):
        m [2,1], v [2,2] -> (E, dE [2,1], d2E [2,2])."""
        y = float(np.asarray(y).reshape(-1)[0])
        m = np.asarray(m, dtype=np.float64).reshape(2, 1)
        v = np.asarray(v, dtype=np.float64).reshape(2, 2)
        x, w = gauss_hermite(2, self.num_cub)
        v = 0.5 * (v + v.T)
        sp = np.linalg.cholesky(v) @ x + m
        E = np.sum(w * self.log_lik(y, sp))
        g, h = self.grad_hess(y, sp)
        return E, (g @ w)[:, None], h @ w

    def log_likelihood_gradients(self, y, f):
        y = float(np.asarray(y).reshape(-1)[0])
        f = np.asarray(f, dtype=np.float64).reshape(2, 1)
        g, h = self.grad_hess(y, f)
        return self.log_lik(y, f)[0], g[:, 0], h[:, :, 0]
