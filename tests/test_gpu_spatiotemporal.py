"""GPU parity of the spatio-temporal VI step (Markov in time, sparse in space)
against the float64 oracle (oracle/spatiotemporal.py), through the C ABI.

Every case has Nr >= 3 M observations per time point: with fewer, the
latent pseudo precision B^T diag(nat2) B has rank Nr < M and its inverse (the
reference's pseudo variance, with only the 1e-12 jitter) is ill-conditioned in
any precision.

Tolerances (float32 on the device, the d x d scan algebra in float32):
data-space marginal means and variances and the latent posterior 5e-4
(normwise relative), energy 1e-5 relative."""
import numpy as np
import pytest

from oracle import kernels as OK
from oracle import likelihoods as OL
from oracle.spatiotemporal import SpatioTemporalKernel as OSTK
from oracle.spatiotemporal import STMarkovGP
from tests._cases import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL, ETOL = 5e-4, 1e-5
KERN = {"m12": "Matern12", "m32": "Matern32", "m52": "Matern52"}


def st_case(Nt, g, Nr, lik, seed=0, missing=0.0, tk="m32", sk="m32", lt=3.0, ls=0.4, conditional=None):
    rng = np.random.default_rng(seed)
    z1 = np.linspace(0.1, 0.9, g)
    za, zb = np.meshgrid(z1, z1)
    z = np.stack([za.ravel(), zb.ravel()], 1)
    X = np.sort(rng.uniform(0, Nt / 2.0, Nt))
    R = rng.uniform(0, 1, [Nt, Nr, 2])
    f = np.sin(3 * R[..., 0] + X[:, None] / 3.0) + 0.5 * np.cos(4 * R[..., 1])
    if lik == "poisson":
        Y = rng.poisson(np.exp(f)).astype(float)
    else:
        Y = f + 0.3 * rng.standard_normal(f.shape)
    if missing:
        Y[rng.uniform(size=Y.shape) < missing] = np.nan
    return dict(z=z, X=X, R=R, Y=Y, lik=lik, tk=tk, sk=sk, lt=lt, ls=ls, cond=conditional)


def _models(c):
    import bayesnewton_gb300 as bnx
    K = bnx.kernels
    tk = getattr(K, KERN[c["tk"]])(1.3, c["lt"])
    sk = getattr(K, KERN[c["sk"]])(0.9, c["ls"])
    gk = K.SpatioTemporalKernel(tk, sk, z=c["z"], conditional=c["cond"])
    gl = bnx.likelihoods.Poisson() if c["lik"] == "poisson" else bnx.likelihoods.Gaussian(0.2)
    ok = OSTK(getattr(OK, KERN[c["tk"]])(1.3, c["lt"]), getattr(OK, KERN[c["sk"]])(0.9, c["ls"]), c["z"])
    ol = OL.Poisson() if c["lik"] == "poisson" else OL.Gaussian(0.2)
    gm = bnx.models.MarkovVariationalGP(gk, gl, c["X"], c["Y"], R=c["R"])
    om = STMarkovGP(ok, ol, c["X"], c["R"], c["Y"], parallel=True)
    if c["cond"] == "DTC":
        om.Cd = np.zeros_like(om.Cd)
    return gm, om


def _check(gm, om):
    mf, vf = om.conditional_posterior_to_data()
    assert rel_err(gm.data_mean.cpu(), mf) < TOL
    assert rel_err(gm.data_variance.cpu(), vf) < TOL
    assert rel_err(gm.posterior_mean.cpu(), om.posterior_mean) < TOL
    assert rel_err(gm.posterior_variance.cpu(), om.posterior_variance) < TOL
    e_g, e_o = gm.energy(), om.energy()
    assert abs(e_g - e_o) <= ETOL * max(1.0, abs(e_o)), (e_g, e_o)


@pytest.mark.parametrize("lik", ["poisson", "gaussian"])
def test_st_two_steps(lik):
    c = st_case(13, 3, 30, lik)
    gm, om = _models(c)
    for _ in range(2):
        gm.inference(lr=1.0)
        om.inference(lr=1.0)
    _check(gm, om)
    assert gm.status() == 0


@pytest.mark.parametrize("tk,sk", [("m12", "m52"), ("m52", "m12"), ("m32", "m32")])
def test_st_matern_orders(tk, sk):
    c = st_case(20, 4, 50, "poisson", seed=1, tk=tk, sk=sk)
    gm, om = _models(c)
    gm.inference(lr=0.7)
    om.inference(lr=0.7)
    _check(gm, om)


@pytest.mark.parametrize("Nt", [1, 2, 3, 64])
def test_st_edge_lengths_missing(Nt):
    c = st_case(Nt, 3, 30, "gaussian", seed=2, missing=0.15 if Nt > 2 else 0.0)
    gm, om = _models(c)
    gm.inference(lr=1.0)
    om.inference(lr=1.0)
    _check(gm, om)


def test_st_dtc_conditional_and_hyperparameter_change():
    c = st_case(16, 3, 30, "poisson", seed=3, conditional="DTC")
    gm, om = _models(c)
    gm.inference(lr=1.0)
    om.inference(lr=1.0)
    _check(gm, om)
    gm.kernel.temporal_kernel.lengthscale = 1.7
    om.kernel.temporal_kernel.lengthscale = 1.7
    gm.inference(lr=1.0)
    om.inference(lr=1.0)
    _check(gm, om)


def test_st_larger_grid():
    """M = 49 inducing inputs (state dim 98), Nt = 100, Nr = 150."""
    c = st_case(100, 7, 150, "poisson", seed=4, lt=8.0, ls=0.25)
    gm, om = _models(c)
    for _ in range(2):
        gm.inference(lr=1.0)
        om.inference(lr=1.0)
    _check(gm, om)


@pytest.mark.parametrize("tk,lik", [("m32", "poisson"), ("m52", "gaussian"), ("m12", "poisson")])
def test_st_predict(tk, lik):
    """Prediction at new times (before, between, on and after the training times)
    and new spatial inputs against the oracle's predict (basemodels.py:766-816),
    itself pinned to the dense GP (tests/test_oracle_invariants.py)."""
    c = st_case(24, 3, 30, lik, seed=4, tk=tk)
    gm, om = _models(c)
    for _ in range(2):
        gm.inference(lr=1.0)
        om.inference(lr=1.0)
    rng = np.random.default_rng(9)
    X = c["X"]
    Xt = np.concatenate([rng.uniform(X[0] - 3, X[-1] + 3, 10), X[[0, 5, 23]]])
    Rt = rng.uniform(0, 1, [Xt.shape[0], 7, 2])
    m_g, v_g = gm.predict(Xt, Rt)
    m_o, v_o = om.predict(Xt, Rt)
    assert rel_err(m_g.cpu(), m_o) < TOL
    assert rel_err(v_g.cpu(), v_o) < TOL
    # at the training inputs the prediction is the data-space posterior (up to the
    # bridge's 1e-8 jitter)
    m_t, v_t = gm.predict()
    mf, vf = om.conditional_posterior_to_data()
    assert rel_err(m_t.cpu(), mf) < 2 * TOL
    assert rel_err(v_t.cpu(), vf) < 2 * TOL
