"""GPU parity of the fused Markov-GP inference step (sites + filter + smoother +
energy) against the float64 oracle model, through the C ABI.

Tolerances: float64 1e-8 relative on posterior means / variances and energy;
float32 2e-4 on posterior means and variances (normwise) and 1e-5 relative on
the energy."""
import numpy as np
import pytest

from oracle import models as OM
from tests._cases import lik_pair, prior_pair, rel_err, series

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {torch.float64: (1e-8, 1e-8), torch.float32: (2e-4, 1e-5)}


def _compare(gm, om, dtype):
    tol, etol = TOL[dtype]
    assert rel_err(gm.posterior_mean.cpu(), om.posterior_mean) < tol
    assert rel_err(gm.posterior_variance.cpu(), om.posterior_variance) < tol


def _run(prior, lik, method, N, dtype, parallel, steps=2, lr=1.0, missing=0.0, spt=0, power=1.0,
         duplicates=False, seed=0):
    import bayesnewton_gb300 as bnx
    ok, gk = prior_pair(prior)
    ol, gl = lik_pair(lik)
    x, y = series(N, lik, seed=seed, missing=missing, duplicates=duplicates)
    cls = {"vi": bnx.models.MarkovVariationalGP, "newton": bnx.models.MarkovNewtonGP,
           "ep": bnx.models.MarkovExpectationPropagationGP,
           "pl": bnx.models.MarkovPosteriorLinearisationGP}[method]
    kw = dict(power=power) if method == "ep" else {}
    gm = cls(gk, gl, x, y, parallel=parallel, dtype=dtype, steps_per_thread=spt, **kw)
    om = OM.MarkovGP(ok, ol, x, y)
    for _ in range(steps):
        gm.inference(lr=lr)
        om.inference(lr=lr, method=method, power=power)
    _compare(gm, om, dtype)
    e_g, e_o = gm.energy(), om.energy(method, power)
    assert abs(e_g - e_o) <= TOL[dtype][1] * max(1.0, abs(e_o)), (e_g, e_o)
    return gm, om


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("parallel", [True, False])
@pytest.mark.parametrize("lik", ["gaussian", "logit", "probit", "poisson"])
def test_vi_step(dtype, parallel, lik):
    _run("m52", lik, "vi", 300, dtype, parallel)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_vi_sum_kernel_long(dtype):
    # several blocks and several aggregates per thread of the block scans
    _run("sum52_32", "logit", "vi", 6000, dtype, True, steps=2, spt=4)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("method", ["newton", "ep"])
@pytest.mark.parametrize("lik", ["gaussian", "logit", "poisson"])
def test_newton_ep_step(dtype, method, lik):
    _run("m52", lik, method, 200, dtype, True, lr=0.8, power=0.7 if method == "ep" else 1.0)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("parallel", [True, False])
@pytest.mark.parametrize("lik", ["gaussian", "logit", "probit", "poisson"])
def test_posterior_linearisation_step(dtype, parallel, lik):
    _run("m52", lik, "pl", 300, dtype, parallel, lr=0.8, missing=0.1 if lik != "poisson" else 0.0)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("link", ["hetero_exp", "hetero_softplus"])
def test_heteroscedastic_two_latents(dtype, link):
    _run("ind52_52", link, "vi", 150, dtype, True, steps=2)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("N", [1, 2, 3, 129])
def test_edge_sizes_missing_duplicates(dtype, N):
    _run("m32", "gaussian", "vi", N, dtype, True, missing=0.2 if N > 3 else 0.0, duplicates=True)


def test_energy_equals_exact_marginal_likelihood():
    """Known answer (tests/test_vs_exact_marg_lik.py:41-59 of the reference): after
    one lr=1 VI step with a Gaussian likelihood the energy is -log N(y | 0, K + s2 I)."""
    import bayesnewton_gb300 as bnx
    from oracle import kernels as OK
    x, y = series(60, "gaussian", seed=3)
    m = bnx.models.MarkovVariationalGP(bnx.kernels.Matern52(1.5, 2.5), bnx.likelihoods.Gaussian(0.5), x, y,
                                       dtype=torch.float64)
    m.inference(lr=1.0)
    Ky = OK.Matern52(1.5, 2.5)(x, x) + 0.5 * np.eye(60)
    L = np.linalg.cholesky(Ky)
    exact = -0.5 * y @ np.linalg.solve(Ky, y) - np.sum(np.log(np.diag(L))) - 30 * np.log(2 * np.pi)
    assert abs(m.energy() + exact) < 1e-8


def test_hyperparameter_change_refreshes_posterior():
    import bayesnewton_gb300 as bnx
    from oracle import kernels as OK
    from oracle import likelihoods as OL
    x, y = series(200, "logit", seed=9)
    k = bnx.kernels.Matern52(1.0, 1.0)
    gm = bnx.models.MarkovVariationalGP(k, bnx.likelihoods.Bernoulli("logit"), x, y, dtype=torch.float64)
    om = OM.MarkovGP(OK.Matern52(1.0, 1.0), OL.Bernoulli("logit"), x, y)
    gm.inference(1.0)
    om.inference(1.0)
    k.lengthscale = 2.0
    om.kernel.lengthscale = 2.0
    gm.inference(1.0)
    om.inference(1.0)
    _compare(gm, om, torch.float64)
    assert abs(gm.energy() - om.energy()) < 1e-8 * abs(om.energy())


def test_float32_overflowing_site_keeps_old_parameters():
    """A count far above its prior (y = 600 at a Poisson site) makes the first
    lr=1 VI step overshoot to a posterior mean near 120, whose rate exp(120)
    is finite in float64 (where the library matches the oracle) but beyond the
    float32 range, and whose neighbours' site precisions (up to ~1e19) are far
    beyond what the float32 covariance update resolves: the float32 step keeps
    the non-finite sites (BN_STATUS_SITE_KEPT), scales the over-precise ones back
    (BN_STATUS_SITE_CLAMPED), and the posterior stays finite."""
    import bayesnewton_gb300 as bnx
    from oracle import kernels as OK, likelihoods as OL
    rng = np.random.default_rng(7)
    N = 2000
    x = np.sort(rng.uniform(0.0, 2000.0, N))
    y = rng.poisson(1.0, N).astype(float)
    y[N // 2] = 600.0
    om = OM.MarkovGP(OK.Matern32(1.0, 4.0), OL.Poisson(), x, y)
    g64 = bnx.models.MarkovVariationalGP(bnx.kernels.Matern32(1.0, 4.0), bnx.likelihoods.Poisson(), x, y,
                                         dtype=torch.float64)
    g32 = bnx.models.MarkovVariationalGP(bnx.kernels.Matern32(1.0, 4.0), bnx.likelihoods.Poisson(), x, y,
                                         dtype=torch.float32)
    for i in range(3):
        om.inference(lr=1.0, method="vi")
        g64.inference(lr=1.0)
        g32.inference(lr=1.0)
        if i == 0:
            assert om.posterior_mean.max() > 100.0  # the overshoot is the algorithm's own
    assert rel_err(g64.posterior_mean.cpu(), om.posterior_mean) < 1e-8
    from bayesnewton_gb300 import _lib
    guard = _lib.STATUS_SITE_KEPT | _lib.STATUS_SITE_CLAMPED
    assert g64.status() & guard == 0
    assert g32.status() & guard
    assert torch.isfinite(g32.posterior_mean).all() and torch.isfinite(g32.posterior_variance).all()
    assert (g32.posterior_variance > 0).all()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("method", ["vi", "newton"])
def test_mean_field_models(dtype, method):
    """MarkovVariationalMeanFieldGP / MarkovNewtonMeanFieldGP against the oracle's
    mean-field filter and smoother (block-diagonal latent covariances)."""
    import bayesnewton_gb300 as bnx
    ok, gk = prior_pair("ind52_52")
    ol, gl = lik_pair("hetero_exp")
    x, y = series(150, "hetero_exp", seed=3)
    cls = {"vi": bnx.models.MarkovVariationalMeanFieldGP, "newton": bnx.models.MarkovNewtonMeanFieldGP}[method]
    gm = cls(gk, gl, x, y, dtype=dtype)
    om = OM.MarkovMeanFieldGP(ok, ol, x, y)
    for _ in range(2):
        gm.inference(lr=0.8)
        om.inference(lr=0.8, method=method)
    _compare(gm, om, dtype)
    e_g, e_o = gm.energy(), om.energy(method)
    assert abs(e_g - e_o) <= TOL[dtype][1] * max(1.0, abs(e_o)), (e_g, e_o)
    with pytest.raises(ValueError):
        cls(bnx.kernels.Matern52(1.0, 1.0), bnx.likelihoods.Gaussian(0.1), x, y)


def test_checkpoint_resume(tmp_path):
    """save() after two steps, load() into a fresh model (other hyperparameters,
    initial sites): the next step of both models is identical."""
    import bayesnewton_gb300 as bnx
    _, gk = prior_pair("sum52_32")
    _, gl = lik_pair("logit")
    x, y = series(500, "logit", seed=8)
    a = bnx.models.MarkovVariationalGP(gk, gl, x, y, dtype=torch.float64)
    for _ in range(2):
        a.inference(lr=1.0)
    a.kernel.components()[0].lengthscale = 1.7
    path = tmp_path / "state.npz"
    a.save(str(path))
    K = bnx.kernels
    b = bnx.models.MarkovVariationalGP(K.Sum([K.Matern52(1.0, 1.0), K.Matern32(1.0, 1.0)]),
                                       bnx.likelihoods.Bernoulli("logit"), x, y, dtype=torch.float64)
    b.load(str(path))
    for m in (a, b):
        m.inference(lr=1.0)
    assert rel_err(a.posterior_mean.cpu(), b.posterior_mean.cpu()) < 1e-12
    assert abs(a.energy() - b.energy()) <= 1e-12 * abs(a.energy())

