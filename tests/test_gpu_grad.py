"""GPU parity of the hyperparameter gradient of the VI energy against the float64
oracle, whose gradient is central differences of its restated energy with the
sites and the stored posterior held fixed (what objax.GradValues(model.energy)
differentiates in the reference; the oracle's dense-GP and Markov-GP gradients
agree, as tests/test_gp_vs_markovgp_reg.py:77-118 of the reference checks).

The library's gradient is analytic (Fisher's identity over a filter + smoother
pass, float64 per-step arithmetic).  Tolerances: float64 1e-6 relative to the
largest component (the oracle's central differences are good to ~1e-9); float32
2e-4 (the float32 smoothed states the gradient starts from)."""
import numpy as np
import pytest

from oracle import models as OM
from tests._cases import lik_pair, prior_pair, series

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-6, torch.float32: 2e-4}


def _check(gm, om, dtype):
    e_g, g = gm.energy_and_grad()
    g_g = np.array(list(g.values()))
    g_o = OM.energy_gradient_fd(om)
    assert g_g.shape == g_o.shape
    err = np.max(np.abs(g_g - g_o)) / max(np.max(np.abs(g_o)), 1e-12)
    assert err < TOL[dtype], (g_g, g_o)
    return g


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("parallel", [True, False])
@pytest.mark.parametrize("prior,lik", [("m52", "gaussian"), ("sum52_32", "logit"), ("m32", "poisson"),
                                       ("m12", "gaussian"), ("ind52_52", "hetero_exp")])
def test_energy_gradient_matches_oracle(dtype, parallel, prior, lik):
    import bayesnewton_gb300 as bnx
    ok, gk = prior_pair(prior)
    ol, gl = lik_pair(lik)
    x, y = series(250, lik, seed=2, duplicates=True)
    gm = bnx.models.MarkovVariationalGP(gk, gl, x, y, parallel=parallel, dtype=dtype)
    om = OM.MarkovGP(ok, ol, x, y)
    # at the initial sites (the reference test's state), then after two steps
    om.update_posterior()
    _check(gm, om, dtype)
    for _ in range(2):
        gm.inference(lr=0.8)
        om.inference(lr=0.8)
    _check(gm, om, dtype)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("method,lik", [("newton", "gaussian"), ("newton", "logit"), ("ep", "gaussian"),
                                        ("ep", "probit"), ("pl", "gaussian"), ("pl", "poisson")])
def test_energy_gradient_other_methods(dtype, method, lik):
    """Newton, EP (power 0.7) and PL energies: the same log Z term, their own
    likelihood terms (log p(y | m); lZ at the cavity over the power)."""
    import bayesnewton_gb300 as bnx
    ok, gk = prior_pair("sum52_32")
    ol, gl = lik_pair(lik)
    x, y = series(220, lik, seed=6, duplicates=True)
    power = 0.7 if method == "ep" else 1.0
    cls = {"newton": bnx.models.MarkovNewtonGP, "ep": bnx.models.MarkovExpectationPropagationGP,
           "pl": bnx.models.MarkovPosteriorLinearisationGP}[method]
    kw = dict(power=power) if method == "ep" else {}
    gm = cls(gk, gl, x, y, dtype=dtype, **kw)
    om = OM.MarkovGP(ok, ol, x, y)
    for _ in range(2):
        gm.inference(lr=0.7)
        om.inference(lr=0.7, method=method, power=power)
    e_g, g = gm.energy_and_grad()
    g_g = np.array(list(g.values()))
    g_o = OM.energy_gradient_fd(om, method=method, power=power)
    err = np.max(np.abs(g_g - g_o)) / max(np.max(np.abs(g_o)), 1e-12)
    assert err < TOL[dtype], (g_g, g_o)


def test_energy_gradient_with_missing_data():
    import bayesnewton_gb300 as bnx
    ok, gk = prior_pair("m52")
    ol, gl = lik_pair("gaussian")
    x, y = series(300, "gaussian", seed=3, missing=0.1)
    gm = bnx.models.MarkovVariationalGP(gk, gl, x, y, dtype=torch.float64)
    om = OM.MarkovGP(ok, ol, x, y)
    gm.inference(lr=1.0)
    om.inference(lr=1.0)
    _check(gm, om, torch.float64)


def test_gradient_equals_exact_marginal_likelihood_gradient():
    """Known answer: with a Gaussian likelihood, after one lr=1 VI step the sites
    are the likelihood itself and q is the exact posterior, so the energy is
    -log N(y | 0, K + s2 I) (tests/test_vs_exact_marg_lik.py:41-59 of the
    reference) and, q being optimal, its gradient at fixed q and sites is minus the
    gradient of that log marginal likelihood: 1/2 tr((a a^T - Ky^-1) dKy), a = Ky^-1 y.
    Also checks the softplus chain rule of transformed=True."""
    import math
    import bayesnewton_gb300 as bnx
    from oracle import kernels as OK
    var_f, len_f, var_y = 1.3, 2.2, 0.25
    x, y = series(200, "gaussian", seed=4)
    gm = bnx.models.MarkovVariationalGP(bnx.kernels.Matern52(var_f, len_f), bnx.likelihoods.Gaussian(var_y), x, y,
                                        dtype=torch.float64)
    gm.inference(lr=1.0)
    _, g = gm.energy_and_grad()
    _, gt = gm.energy_and_grad(transformed=True)

    def kmat(v, l):
        return OK.Matern52(v, l)(x[:, None], x[:, None])

    Ky = kmat(var_f, len_f) + var_y * np.eye(x.shape[0])
    a = np.linalg.solve(Ky, y)
    W = np.outer(a, a) - np.linalg.inv(Ky)
    h = 1e-6 * len_f
    dK = {"kernel.0.variance": kmat(var_f, len_f) / var_f,
          "kernel.0.lengthscale": (kmat(var_f, len_f + h) - kmat(var_f, len_f - h)) / (2 * h),
          "likelihood.variance": np.eye(x.shape[0])}
    for name, d in dK.items():
        exact = -0.5 * np.sum(W * d)
        assert abs(g[name] - exact) <= 1e-6 * max(1.0, abs(exact)), (name, g[name], exact)
    for (name, obj, attr) in gm.hyperparameters():
        v = getattr(obj, attr)
        assert abs(gt[name] - g[name] * (1 - math.exp(-v))) <= 1e-12 * max(1.0, abs(g[name]))


def test_energy_gradient_long_series_float32():
    """N = 1e6 (the step's workload size): float32 gradient against the float64
    engine's on the same sites (the oracle is too slow at this size)."""
    import bayesnewton_gb300 as bnx
    K = bnx.kernels
    N = 1_000_000
    rng = np.random.default_rng(0)
    x = np.sort(rng.uniform(0.0, 1e4, N))
    y = (rng.uniform(size=N) < 1.0 / (1.0 + np.exp(-2.0 * np.sin(x / 5.0)))).astype(float)
    mk = lambda dt: bnx.models.MarkovVariationalGP(K.Sum([K.Matern52(1.0, 1.0), K.Matern32(1.0, 1.0)]),
                                                   bnx.likelihoods.Bernoulli("logit"), x, y, dtype=dt)
    g32, g64 = mk(torch.float32), mk(torch.float64)
    for m in (g32, g64):
        m.inference(lr=1.0)
    # same sites in both
    g64._nat1.copy_(g32._nat1.double())
    g64._nat2.copy_(g32._nat2.double())
    g64._stale = True
    _, a = g32.energy_and_grad()
    _, b = g64.energy_and_grad()
    va, vb = np.array(list(a.values())), np.array(list(b.values()))
    assert np.max(np.abs(va - vb)) / np.max(np.abs(vb)) < 1e-3, (va, vb)
