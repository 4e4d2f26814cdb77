"""Oracle Gauss-Hermite cubature (float64 numpy restatement).

Nodes and weights come from ``numpy.polynomial.hermite.hermgauss``, the same
routine the reference calls (bayesnewton/cubature.py:6, 70), arranged as a
tensor-product grid whose first coordinate varies slowest
(cubature.py:56-84).
"""
import itertools

import numpy as np
from numpy.polynomial.hermite import hermgauss


def mvhermgauss(H, D):
    """Tensor-product GH grid: x [H**D, D], w [H**D] (cubature.py:56-73)."""
    gh_x, gh_w = hermgauss(H)
    x = np.array(list(itertools.product(*(gh_x,) * D)))
    w = np.prod(np.array(list(itertools.product(*(gh_w,) * D))), 1)
    return x, w


def gauss_hermite(dim=1, num_quad_pts=20):
    """Sigma points [dim, n**dim] scaled by sqrt(2), weights scaled by pi^(-dim/2)
    (cubature.py:76-84)."""
    x, w = mvhermgauss(num_quad_pts, dim)
    return np.sqrt(2.0) * x.T, w.T * np.pi ** (-0.5 * dim)


def variational_expectation_cubature(loglik, y, m, v, num_quad_pts=20):
    """Score-function cubature for one scalar site (cubature.py:198-246).

    loglik(y, f) evaluates log p(y|f) at an array of f.
    Returns (E, dE/dm, d2E/dm2) with
      E       = sum_i w_i log p(y | sqrt(v) x_i + m)
      dE/dm   = sum_i w_i (f_i - m)/v * log p
      d2E/dm2 = 2 sum_i w_i [0.5 (f_i - m)^2 / v^2 - 0.5 / v] * log p
    """
    x, w = gauss_hermite(1, num_quad_pts)
    x = x[0]
    sp = np.sqrt(v) * x + m
    wl = w * loglik(y, sp)
    E = np.sum(wl)
    invv = 1.0 / v
    dE = np.sum(invv * (sp - m) * wl)
    dEdv = np.sum((0.5 * (invv ** 2 * (sp - m) ** 2) - 0.5 * invv) * wl)
    return E, dE, 2.0 * dEdv


def moment_match_cubature(loglik, y, cav_mean, cav_cov, power=1.0, num_quad_pts=20):
    """Log partition function and its mean derivatives (cubature.py:310-371).

    cav_mean [D, 1], cav_cov [D, D]; loglik(y, f) takes f [D, Q] and returns [Q].
    """
    D = cav_mean.shape[0]
    x, w = gauss_hermite(D, num_quad_pts)
    cav_cov = 0.5 * (cav_cov + cav_cov.T)
    L = np.linalg.cholesky(cav_cov)
    sp = L @ np.atleast_2d(x) + cav_mean
    wle = w * np.exp(power * loglik(y, sp))
    Z = np.sum(wle)
    lZ = np.log(np.maximum(Z, 1e-8))
    Zinv = 1.0 / np.maximum(Z, 1e-8)
    invC = np.linalg.inv(cav_cov)
    diff = sp - cav_mean                      # [D, Q]
    sdiff = invC @ diff                       # [D, Q]
    dZ = np.sum(sdiff * wle, axis=1)[:, None]
    d2Z = np.einsum('iq,jq,q->ij', sdiff, sdiff, wle) - invC * np.sum(wle)
    dlZ = Zinv * dZ
    d2lZ = -dlZ @ dlZ.T + Zinv * d2Z
    return lZ, dlZ, d2lZ
