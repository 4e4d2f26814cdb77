"""Oracle SDE priors (float64 numpy restatement).

Follows bayesnewton/kernels.py: the generic ``Kernel.state_transition`` = expm(F dt)
(kernels.py:63-67), Matern12 (:123-169), Matern32 (:175-230), Matern52 (:233-300),
Matern72 (:303-382), Independent (:1499-1616) and Sum (:1624-1663).

``state_transition`` accepts a scalar dt or a 1-D array of dt values and then
returns a stacked [N, d, d] array (the reference vmaps the scalar form).
Hyperparameters are held as plain values; the reference stores them through a
softplus transform, which round-trips to the same value up to ~1e-16.
"""
import numpy as np
from scipy.linalg import block_diag, expm


def _as_inputs(X):
    X = np.asarray(X, dtype=np.float64)
    return X[:, None] if X.ndim < 2 else X


def _r(X, X2, ell):
    X, X2 = _as_inputs(X), _as_inputs(X2)
    d = (X[:, None, :] / ell - X2[None, :, :] / ell)
    r2 = np.sum(d * d, axis=-1)
    # kernels.py:106-108 clips r2 at 1e-36 before the square root
    return np.sqrt(np.maximum(r2, 1e-36))


def _stack(A, dt):
    return A if np.ndim(dt) else A[0]


class StationaryKernel:
    state_dim = None
    name = None

    def __init__(self, variance=1.0, lengthscale=1.0):
        self.variance = float(variance)
        self.lengthscale = float(lengthscale)

    def __call__(self, X, X2):
        return self.K(X, X2)

    def K(self, X, X2):
        return self.K_r(_r(X, X2, self.lengthscale))

    def measurement_model(self):
        H = np.zeros([1, self.state_dim])
        H[0, 0] = 1.0
        return H


class Matern12(StationaryKernel):
    state_dim = 1
    name = "matern12"

    def K_r(self, r):
        return self.variance * np.exp(-r)

    def stationary_covariance(self):
        return np.array([[self.variance]])

    def feedback_matrix(self):
        return np.array([[-1.0 / self.lengthscale]])

    def state_transition(self, dt):
        dt1 = np.atleast_1d(np.asarray(dt, dtype=np.float64))
        A = np.exp(-dt1 / self.lengthscale)[:, None, None]
        return _stack(A, dt)


class Matern32(StationaryKernel):
    state_dim = 2
    name = "matern32"

    def K_r(self, r):
        s3 = np.sqrt(3.0)
        return self.variance * (1.0 + s3 * r) * np.exp(-s3 * r)

    def stationary_covariance(self):
        return np.array([[self.variance, 0.0],
                         [0.0, 3.0 * self.variance / self.lengthscale ** 2.0]])

    def feedback_matrix(self):
        lam = 3.0 ** 0.5 / self.lengthscale
        return np.array([[0.0, 1.0], [-lam ** 2, -2 * lam]])

    def state_transition(self, dt):
        # kernels.py:216-224
        t = np.atleast_1d(np.asarray(dt, dtype=np.float64))
        lam = np.sqrt(3.0) / self.lengthscale
        e = np.exp(-t * lam)
        A = np.empty([t.shape[0], 2, 2])
        A[:, 0, 0] = e * (t * lam + 1.0)
        A[:, 0, 1] = e * t
        A[:, 1, 0] = e * (-t * lam ** 2)
        A[:, 1, 1] = e * (-t * lam + 1.0)
        return _stack(A, dt)


class Matern52(StationaryKernel):
    state_dim = 3
    name = "matern52"

    def K_r(self, r):
        s5 = np.sqrt(5.0)
        return self.variance * (1.0 + s5 * r + 5.0 / 3.0 * r * r) * np.exp(-s5 * r)

    def stationary_covariance(self):
        v, l = self.variance, self.lengthscale
        kappa = 5.0 / 3.0 * v / l ** 2.0
        return np.array([[v, 0.0, -kappa],
                         [0.0, kappa, 0.0],
                         [-kappa, 0.0, 25.0 * v / l ** 4.0]])

    def feedback_matrix(self):
        lam = 5.0 ** 0.5 / self.lengthscale
        return np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0],
                         [-lam ** 3.0, -3.0 * lam ** 2.0, -3.0 * lam]])

    def state_transition(self, dt):
        # kernels.py:273-286
        t = np.atleast_1d(np.asarray(dt, dtype=np.float64))
        lam = np.sqrt(5.0) / self.lengthscale
        tl = t * lam
        e = np.exp(-tl)
        M = np.empty([t.shape[0], 3, 3])
        M[:, 0, 0] = lam * (0.5 * tl + 1.0)
        M[:, 0, 1] = tl + 1.0
        M[:, 0, 2] = 0.5 * t
        M[:, 1, 0] = -0.5 * tl * lam ** 2
        M[:, 1, 1] = lam * (1.0 - tl)
        M[:, 1, 2] = 1.0 - 0.5 * tl
        M[:, 2, 0] = lam ** 3 * (0.5 * tl - 1.0)
        M[:, 2, 1] = lam ** 2 * (tl - 3)
        M[:, 2, 2] = lam * (0.5 * tl - 2.0)
        A = e[:, None, None] * (t[:, None, None] * M + np.eye(3)[None])
        return _stack(A, dt)


class Matern72(StationaryKernel):
    state_dim = 4
    name = "matern72"

    def K_r(self, r):
        s7 = np.sqrt(7.0)
        return self.variance * (1. + s7 * r + 14. / 5. * r * r + 7. * s7 / 15. * r ** 3) * np.exp(-s7 * r)

    def stationary_covariance(self):
        v, l = self.variance, self.lengthscale
        kappa = 7.0 / 5.0 * v / l ** 2.0
        kappa2 = 9.8 * v / l ** 4.0
        return np.array([[v, 0.0, -kappa, 0.0],
                         [0.0, kappa, 0.0, -kappa2],
                         [-kappa, 0.0, kappa2, 0.0],
                         [0.0, -kappa2, 0.0, 343.0 * v / l ** 6.0]])

    def feedback_matrix(self):
        lam = 7.0 ** 0.5 / self.lengthscale
        return np.array([[0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0],
                         [-lam ** 4.0, -4.0 * lam ** 3.0, -6.0 * lam ** 2.0, -4.0 * lam]])

    def state_transition(self, dt):
        # kernels.py:344-365
        t = np.atleast_1d(np.asarray(dt, dtype=np.float64))
        lam = np.sqrt(7.0) / self.lengthscale
        l2, l3 = lam * lam, lam * lam * lam
        tl = t * lam
        tl2 = tl ** 2
        M = np.empty([t.shape[0], 4, 4])
        M[:, 0, 0] = lam * (1.0 + 0.5 * tl + tl2 / 6.0)
        M[:, 0, 1] = 1.0 + tl + 0.5 * tl2
        M[:, 0, 2] = 0.5 * t * (1.0 + tl)
        M[:, 0, 3] = t ** 2 / 6
        M[:, 1, 0] = -tl2 * lam ** 2.0 / 6.0
        M[:, 1, 1] = lam * (1.0 + 0.5 * tl - 0.5 * tl2)
        M[:, 1, 2] = 1.0 + tl - 0.5 * tl2
        M[:, 1, 3] = t * (0.5 - tl / 6.0)
        M[:, 2, 0] = l3 * tl * (tl / 6.0 - 0.5)
        M[:, 2, 1] = tl * l2 * (0.5 * tl - 2.0)
        M[:, 2, 2] = lam * (1.0 - 2.5 * tl + 0.5 * tl2)
        M[:, 2, 3] = 1.0 - tl + tl2 / 6.0
        M[:, 3, 0] = l2 ** 2 * (tl - 1.0 - tl2 / 6.0)
        M[:, 3, 1] = l3 * (3.5 * tl - 4.0 - 0.5 * tl2)
        M[:, 3, 2] = l2 * (4.0 * tl - 6.0 - 0.5 * tl2)
        M[:, 3, 3] = lam * (1.5 * tl - 3.0 - tl2 / 6.0)
        A = np.exp(-tl)[:, None, None] * (t[:, None, None] * M + np.eye(4)[None])
        return _stack(A, dt)


class FeedbackKernel:
    """A prior given only by (F, Pinf, H): the transition is the generic
    ``A = expm(F dt)`` of bayesnewton/kernels.py:63-67."""

    def __init__(self, F, Pinf, H=None):
        self.F = np.asarray(F, dtype=np.float64)
        self.Pinf = np.asarray(Pinf, dtype=np.float64)
        d = self.F.shape[0]
        if H is None:
            H = np.zeros([1, d])
            H[0, 0] = 1.0
        self.H = np.asarray(H, dtype=np.float64)
        self.state_dim = d
        self.name = "feedback"

    @classmethod
    def of(cls, kernel):
        return cls(kernel.feedback_matrix(), kernel.stationary_covariance(), kernel.measurement_model())

    def stationary_covariance(self):
        return self.Pinf

    def measurement_model(self):
        return self.H

    def feedback_matrix(self):
        return self.F

    def state_transition(self, dt):
        t = np.atleast_1d(np.asarray(dt, dtype=np.float64))
        A = np.stack([expm(self.F * ti) for ti in t])
        return _stack(A, dt)


class Independent:
    """Stacked independent priors, H = block_diag (kernels.py:1499-1616)."""
    name = "independent"

    def __init__(self, kernels):
        self.kernels = list(kernels)
        self.num_kernels = len(self.kernels)
        self.state_dim = sum(k.state_dim for k in self.kernels)

    def __call__(self, X, X2):
        return self.K(X, X2)

    def K(self, X, X2):
        Ks = None
        for i, k in enumerate(self.kernels):
            e = np.zeros(self.num_kernels)
            e[i] = 1.0
            term = np.kron(k.K(X, X2), np.diag(e))
            Ks = term if Ks is None else Ks + term
        return Ks

    def stationary_covariance(self):
        return block_diag(*[k.stationary_covariance() for k in self.kernels])

    def measurement_model(self):
        return block_diag(*[k.measurement_model() for k in self.kernels])

    def feedback_matrix(self):
        return block_diag(*[k.feedback_matrix() for k in self.kernels])

    def state_transition(self, dt):
        parts = [np.atleast_3d(k.state_transition(np.atleast_1d(dt))) for k in self.kernels]
        n = parts[0].shape[0]
        A = np.zeros([n, self.state_dim, self.state_dim])
        o = 0
        for p in parts:
            s = p.shape[-1]
            A[:, o:o + s, o:o + s] = p
            o += s
        return _stack(A, dt)


class Sum(Independent):
    """Sum of priors, H = hstack (kernels.py:1624-1663)."""
    name = "sum"

    def K(self, X, X2):
        return sum(k.K(X, X2) for k in self.kernels)

    def measurement_model(self):
        return np.hstack([k.measurement_model() for k in self.kernels])
