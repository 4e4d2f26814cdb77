"""GPU parity of the infinite-horizon Markov GP (InfiniteHorizonGaussianProcess,
basemodels.py:1257-1308; ops.py:796-1068) against the float64 oracle, through
the C ABI: posterior marginals, energies and the Riccati warm starts after the
reference's call sequence (inference = update_posterior, site update,
update_posterior; energy = a fresh filter), for the homoscedastic (Gaussian, no
missing data) and heteroscedastic (missing data, non-Gaussian) filters.

Tolerances: float64 1e-9 relative; float32 2e-4 on the posterior and 1e-5 on the
energy."""
import numpy as np
import pytest

from oracle import models as OM
from tests._cases import lik_pair, prior_pair, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {torch.float64: (1e-9, 1e-9), torch.float32: (2e-4, 1e-5)}


def _series(N, lik, seed, missing=0.0, step=0.1):
    rng = np.random.default_rng(seed)
    x = np.arange(N) * step + 3.0
    f = np.sin(x / 3.0) + 0.3 * np.cos(x)
    if lik == "gaussian":
        y = f + np.sqrt(0.1) * rng.standard_normal(N)
    elif lik in ("logit", "probit"):
        y = (rng.uniform(size=N) < 1.0 / (1.0 + np.exp(-2.0 * f))).astype(float)
    else:
        y = rng.poisson(np.exp(f)).astype(float)
    if missing:
        y[rng.uniform(size=N) < missing] = np.nan
    return x, y


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("prior,lik,missing,method", [
    ("m52", "gaussian", 0.0, "vi"), ("m32", "gaussian", 0.1, "vi"), ("sum52_32", "logit", 0.0, "vi"),
    ("m52", "poisson", 0.0, "vi"), ("m32", "probit", 0.0, "newton"), ("m52", "logit", 0.1, "ep"),
    ("m32", "poisson", 0.0, "pl")])
def test_infinite_horizon_matches_oracle(dtype, prior, lik, missing, method):
    import bayesnewton_gb300 as bnx
    IH = bnx.infinite_horizon
    ok, gk = prior_pair(prior)
    ol, gl = lik_pair(lik)
    x, y = _series(3000 if dtype == torch.float64 else 5000, lik, seed=1, missing=missing)
    cls = {"vi": IH.InfiniteHorizonVariationalGP, "newton": IH.InfiniteHorizonNewtonGP,
           "ep": IH.InfiniteHorizonExpectationPropagationGP, "pl": IH.InfiniteHorizonPosteriorLinearisationGP}[method]
    gm = cls(gk, gl, x, y, dtype=dtype)
    om = OM.InfiniteHorizonGP(ok, ol, x, y)
    tol, etol = TOL[dtype]
    for _ in range(3):
        gm.inference(lr=0.9)
        om.inference(lr=0.9, method=method)
        assert rel_err(gm.posterior_mean.cpu(), om.posterior_mean) < tol
        assert rel_err(gm.posterior_variance.cpu(), om.posterior_variance) < tol
        e_g, e_o = gm.energy(), om.energy(method)
        assert abs(e_g - e_o) <= etol * max(1.0, abs(e_o)), (e_g, e_o)
    f_g, s_g = gm.dare_state()
    assert rel_err(f_g, om.dare_init_filter) < tol
    assert rel_err(s_g, om.dare_init_smoother) < tol


def test_infinite_horizon_long_series_equals_full_model_in_the_middle():
    """N = 1e6 float32, Gaussian likelihood, 200 Riccati steps: in the steady state
    the infinite-horizon posterior equals the full Markov GP's (float32 engines
    both)."""
    import bayesnewton_gb300 as bnx
    _, gk = prior_pair("m32")
    _, gl = lik_pair("gaussian")
    x, y = _series(1_000_000, "gaussian", seed=2, step=0.05)
    ih = bnx.infinite_horizon.InfiniteHorizonVariationalGP(gk, gl, x, y, dare_iters=200)
    full = bnx.models.MarkovVariationalGP(gk, gl, x, y)
    ih.inference(lr=1.0)
    full.inference(lr=1.0)
    a = ih.posterior_mean[1000:-1000].cpu().numpy()
    b = full.posterior_mean[1000:-1000].cpu().numpy()
    assert rel_err(a, b) < 1e-4
    va = ih.posterior_variance[1000:-1000].cpu().numpy()
    vb = full.posterior_variance[1000:-1000].cpu().numpy()
    assert rel_err(va, vb) < 1e-3


@pytest.mark.parametrize("N", [2, 3, 5])
def test_infinite_horizon_tiny_series(N):
    import bayesnewton_gb300 as bnx
    ok, gk = prior_pair("m32")
    ol, gl = lik_pair("logit")
    x, y = _series(N, "logit", seed=3)
    gm = bnx.infinite_horizon.InfiniteHorizonVariationalGP(gk, gl, x, y, dtype=torch.float64)
    om = OM.InfiniteHorizonGP(ok, ol, x, y)
    for _ in range(2):
        gm.inference(lr=1.0)
        om.inference(lr=1.0)
    assert rel_err(gm.posterior_mean.cpu(), om.posterior_mean) < 1e-9
    assert abs(gm.energy() - om.energy()) <= 1e-9 * max(1.0, abs(om.energy()))


def test_infinite_horizon_rejects_uneven_times():
    import bayesnewton_gb300 as bnx
    _, gk = prior_pair("m32")
    _, gl = lik_pair("gaussian")
    with pytest.raises(ValueError):
        bnx.infinite_horizon.InfiniteHorizonVariationalGP(gk, gl, np.array([0.0, 1.0, 2.5]), np.zeros(3))
    with pytest.raises(ValueError):
        bnx.infinite_horizon.InfiniteHorizonVariationalGP(gk, gl, np.array([0.0]), np.zeros(1))
