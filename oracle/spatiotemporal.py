"""Oracle spatio-temporal Markov GP (float64 numpy restatement; TEST
INFRASTRUCTURE: the parity reference of the library's spatio-temporal path,
never part of it).

Follows bayesnewton/kernels.py SpatioTemporalKernel (:385-586: the separable
prior with M spatial inducing inputs z, state x(t) = [x_1(t), ..., x_M(t)] of M
independent temporal processes, A = kron(I_M, A_t), Pinf = kron(I_M, Pinf_t),
H = kron(I_M, H_t); the spatial conditional f(t, R) | u(t) ~ N(B u(t), C) with
B = Krz Kzz^-1 Lzz and the 'Full' conditional covariance
C = k_t(t, t) (Krr - Krz Kzz^-1 Kzr), :476-505) and bayesnewton/basemodels.py
MarkovGaussianProcess in its spatio-temporal case (compute_full_pseudo_lik
:676-687 with the 1e-12 jitter, update_posterior :689-706, compute_kl :708-724,
compute_log_lik :726-741, conditional_posterior_to_data :743-764, predict :766-816), with the VI
site update and energy of bayesnewton/inference.py (:170-222).

Data layout (the reference's input_admin for spatio-temporal inputs): time
points X [Nt], spatial inputs R [Nt, Nr, 2] and observations Y [Nt, Nr]; every
time point carries Nr observations.  Sites live in data space, one scalar
(nat1, nat2) per observation (the reference's [Nt, Nr, Nr] site covariance is
diagonal because its VI Hessian is), so they are held as [Nt, Nr] arrays.
"""
import math

import numpy as np

from . import ops

LOG2PI = math.log(2 * math.pi)


class SpatioTemporalKernel:
    """temporal_kernel (a Markov kernel) x spatial_kernel at inducing inputs z [M, D]."""

    def __init__(self, temporal_kernel, spatial_kernel, z):
        self.temporal_kernel = temporal_kernel
        self.spatial_kernel = spatial_kernel
        self.z = np.asarray(z, dtype=np.float64)
        if self.z.ndim < 2:
            self.z = self.z[:, None]
        self.M = self.z.shape[0]

    @property
    def state_dim(self):
        return self.M * self.temporal_kernel.state_dim

    def stationary_covariance(self):
        return np.kron(np.eye(self.M), self.temporal_kernel.stationary_covariance())

    def measurement_model(self):
        return np.kron(np.eye(self.M), self.temporal_kernel.measurement_model())

    def state_transition(self, dt):
        At = self.temporal_kernel.state_transition(dt)
        if np.ndim(dt):
            return np.stack([np.kron(np.eye(self.M), a) for a in At])
        return np.kron(np.eye(self.M), At)

    def inducing_precision(self):
        """(Kzz^-1, chol(Kzz)) (kernels.py:507-514)."""
        Kzz = self.spatial_kernel(self.z, self.z)
        Lzz = np.linalg.cholesky(Kzz)
        return ops.inv(Kzz), Lzz

    def spatial_conditional(self, X, R):
        """B [Nt, Nr, M], diag(C) [Nt, Nr] (kernels.py:486-505, 'Full'; only the
        diagonal of C enters the VI site update and energy)."""
        Qzz, Lzz = self.inducing_precision()
        B = np.empty([R.shape[0], R.shape[1], self.M])
        Cd = np.empty([R.shape[0], R.shape[1]])
        kt0 = float(self.temporal_kernel.K(np.zeros(1), np.zeros(1))[0, 0])
        for n in range(R.shape[0]):
            Krz = self.spatial_kernel(R[n], self.z)
            K = Krz @ Qzz
            B[n] = K @ Lzz
            Krr_d = np.diag(self.spatial_kernel(R[n], R[n]))
            Cd[n] = kt0 * (Krr_d - np.sum(K * Krz, axis=1))
        return B, Cd


class STMarkovGP:
    """MarkovVariationalGP with a SpatioTemporalKernel (sparse in space)."""

    def __init__(self, kernel, likelihood, X, R, Y, parallel=False):
        X = np.asarray(X, dtype=np.float64).reshape(-1)
        ind = np.argsort(X, kind="stable")
        self.X = X[ind]
        self.R = np.asarray(R, dtype=np.float64)[ind]
        self.Y = np.asarray(Y, dtype=np.float64)[ind]
        self.dt = np.concatenate([[0.0], np.diff(self.X)])
        self.kernel = kernel
        self.likelihood = likelihood
        self.parallel = parallel
        self.Nt, self.Nr = self.Y.shape
        self.M = kernel.M
        # sites start at mean 0, covariance 1e2 (basemodels.py:130-133)
        self.site_nat1 = np.zeros([self.Nt, self.Nr])
        self.site_nat2 = np.full([self.Nt, self.Nr], 1e-2)
        self.posterior_mean = np.zeros([self.Nt, self.M, 1])
        self.posterior_variance = np.tile(np.eye(self.M), [self.Nt, 1, 1])
        self.B, self.Cd = kernel.spatial_conditional(self.X, self.R)

    def compute_full_pseudo_lik(self):
        """basemodels.py:676-687: latent-space pseudo observations."""
        B = self.B
        Bt = np.swapaxes(B, 1, 2)
        nat1 = Bt @ self.site_nat1[..., None]                     # B^T nat1
        nat2 = Bt @ (self.site_nat2[..., None] * B) + 1e-12 * np.eye(self.M)  # B^T diag(nat2) B
        pv = ops.inv(nat2)
        py = pv @ nat1
        return py, pv

    def update_posterior(self):
        py, pv = self.compute_full_pseudo_lik()
        ell, (fm, fP) = ops.kalman_filter(self.dt, self.kernel, py, pv, mask=None, parallel=self.parallel)
        self.last_log_lik = ell
        dts = np.concatenate([self.dt[1:], [0.0]])
        sm, sP, _ = ops.rauch_tung_striebel_smoother(dts, self.kernel, fm, fP, parallel=self.parallel)
        self.posterior_mean, self.posterior_variance = sm, sP

    def conditional_posterior_to_data(self):
        """basemodels.py:743-764: marginal mean and variance of f at each observation."""
        mean_f = (self.B @ self.posterior_mean)[..., 0]
        var_f = np.sum((self.B @ self.posterior_variance) * self.B, axis=2) + self.Cd  # diag(B P B^T) + C
        return mean_f, var_f

    def predict(self, X_test, R_test):
        """basemodels.py:766-816, spatio-temporal case: filter and full smoother with
        gains from the sites, the state at each test time from its two neighbours
        (utils.py:123-138), then f = B H x at the test inputs with the spatial
        conditional (kernels.py:486-505 with predict=True): mean W m, variance
        diag(W P W^T) + diag(C), W = B H.  X_test [Nt*], R_test [Nt*, Nr*, D]."""
        py, pv = self.compute_full_pseudo_lik()
        _, (fm, fP) = ops.kalman_filter(self.dt, self.kernel, py, pv, mask=None, parallel=self.parallel)
        dts = np.concatenate([self.dt[1:], [0.0]])
        sm, sP, G = ops.rauch_tung_striebel_smoother(dts, self.kernel, fm, fP, return_full=True,
                                                     parallel=self.parallel)
        X_aug = np.concatenate([[-1e10], self.X, [1e10]])
        xt = np.asarray(X_test, dtype=np.float64).reshape(-1)
        m, P = ops.temporal_conditional(X_aug, xt, sm, sP, G, self.kernel)
        H = self.kernel.measurement_model()
        B, Cd = self.kernel.spatial_conditional(xt, np.asarray(R_test, dtype=np.float64))
        W = B @ H
        mean = (W @ m)[..., 0]
        var = np.sum((W @ P) * W, axis=2) + Cd
        return mean, var

    def _ve(self, mean_f, var_f):
        # per observation, NaN = missing (likelihoods.py:363-383)
        lik = self.likelihood
        E = np.zeros_like(mean_f)
        g = np.full_like(mean_f, np.nan)
        h = np.full_like(mean_f, np.nan)
        for n in range(self.Nt):
            for r in range(self.Nr):
                if not np.isnan(self.Y[n, r]):
                    E[n, r], g[n, r], h[n, r] = lik.ve_scalar(self.Y[n, r], mean_f[n, r], var_f[n, r])
        return E, g, h

    def inference(self, lr=1.0, ensure_psd=True):
        """InferenceMixin.inference (inference.py:65-90) with the VI update (:170-195)."""
        self.update_posterior()
        mean_f, var_f = self.conditional_posterior_to_data()
        _, jac, hess = self._ve(mean_f, var_f)
        if ensure_psd:
            hess = -np.where(-hess < 0, 1e-2, -hess)
        hess = np.where(np.isnan(hess), -1e-6, hess)
        jac = np.where(np.isnan(jac), hess * mean_f, jac)
        nat1_n, nat2_n = jac - hess * mean_f, -hess
        self.site_nat1 = (1 - lr) * self.site_nat1 + lr * nat1_n
        self.site_nat2 = (1 - lr) * self.site_nat2 + lr * nat2_n
        self.update_posterior()

    def compute_log_lik(self):
        py, pv = self.compute_full_pseudo_lik()
        ell, _ = ops.kalman_filter(self.dt, self.kernel, py, pv, mask=None, parallel=self.parallel)
        return ell

    def compute_kl(self):
        """basemodels.py:708-724 with gaussian_expected_log_lik (utils.py:510-531)."""
        py, pv = self.compute_full_pseudo_lik()
        ll = self.compute_log_lik()
        tot = 0.0
        for n in range(self.Nt):
            tot += ops.mvn_logpdf(py[n], self.posterior_mean[n], pv[n]) \
                - 0.5 * np.trace(ops.solve(pv[n], self.posterior_variance[n]))
        return tot - ll

    def energy(self):
        """VariationalInference.energy (inference.py:197-222)."""
        mean_f, var_f = self.conditional_posterior_to_data()
        ell, _, _ = self._ve(mean_f, var_f)
        return -(np.nansum(ell) - self.compute_kl())
