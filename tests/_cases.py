"""Shared seeded cases for the parity tests (oracle kernels paired with the
library's kernels)."""
import numpy as np

from oracle import kernels as OK
from oracle import likelihoods as OL


def prior_pair(name):
    import bayesnewton_gb300 as bnx
    K = bnx.kernels
    table = {
        "m12": (OK.Matern12(0.8, 1.3), K.Matern12(0.8, 1.3)),
        "m32": (OK.Matern32(1.2, 0.7), K.Matern32(1.2, 0.7)),
        "m52": (OK.Matern52(1.0, 1.0), K.Matern52(1.0, 1.0)),
        "m72": (OK.Matern72(0.9, 2.0), K.Matern72(0.9, 2.0)),
        "sum52_32": (OK.Sum([OK.Matern52(1.0, 1.5), OK.Matern32(0.5, 4.0)]),
                     K.Sum([K.Matern52(1.0, 1.5), K.Matern32(0.5, 4.0)])),
        # not a compiled layout: runs on the dense single-block (expm) path
        "sum32_12_32": (OK.Sum([OK.Matern32(1.0, 1.5), OK.Matern12(0.3, 2.0), OK.Matern32(0.5, 4.0)]),
                        K.Sum([K.Matern32(1.0, 1.5), K.Matern12(0.3, 2.0), K.Matern32(0.5, 4.0)])),
        "ind52_52": (OK.Independent([OK.Matern52(1.0, 2.0), OK.Matern52(0.7, 5.0)]),
                     K.Independent([K.Matern52(1.0, 2.0), K.Matern52(0.7, 5.0)])),
        "ind32_32": (OK.Independent([OK.Matern32(1.0, 2.0), OK.Matern32(0.7, 5.0)]),
                     K.Independent([K.Matern32(1.0, 2.0), K.Matern32(0.7, 5.0)])),
    }
    return table[name]


def lik_pair(name):
    import bayesnewton_gb300 as bnx
    L = bnx.likelihoods
    table = {
        "gaussian": (OL.Gaussian(0.1), L.Gaussian(0.1)),
        "logit": (OL.Bernoulli("logit"), L.Bernoulli("logit")),
        "probit": (OL.Bernoulli("probit"), L.Bernoulli("probit")),
        "poisson": (OL.Poisson(), L.Poisson()),
        "hetero_exp": (OL.HeteroscedasticNoise("exp"), L.HeteroscedasticNoise("exp")),
        "hetero_softplus": (OL.HeteroscedasticNoise("softplus"), L.HeteroscedasticNoise("softplus")),
    }
    return table[name]


def series(N, lik, seed=0, missing=0.0, span=None, duplicates=False):
    """Seeded synthetic series: x sorted in [0, span], y drawn for the likelihood."""
    rng = np.random.default_rng(seed)
    span = span if span is not None else max(10.0, N / 10.0)
    x = np.sort(rng.uniform(0.0, span, N))
    if duplicates and N > 4:
        x[N // 2] = x[N // 2 - 1]
    f = np.sin(x / 3.0) + 0.3 * np.cos(x)
    if lik == "gaussian":
        y = f + np.sqrt(0.1) * rng.standard_normal(N)
    elif lik in ("logit", "probit"):
        y = (rng.uniform(size=N) < 1.0 / (1.0 + np.exp(-2.0 * f))).astype(float)
    elif lik == "poisson":
        y = rng.poisson(np.exp(f)).astype(float)
    else:
        y = f + np.exp(0.3 * np.cos(x / 2.0)) * rng.standard_normal(N)
    if missing > 0:
        y[rng.uniform(size=N) < missing] = np.nan
    return x, y


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def elem_rel_err(a, b, floor=1e-3):
    """Elementwise relative error max |a - b| / max(|b|, floor * max |b|): each
    entry against its own size, entries below `floor` of the largest measured
    against that floor (so values crossing zero do not divide by ~0)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.maximum(np.abs(b), floor * max(np.max(np.abs(b)), 1e-300))
    return float(np.max(np.abs(a - b) / scale))
