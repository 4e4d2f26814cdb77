"""GPU parity of prediction at new times (MarkovGaussianProcess.predict,
utils.temporal_conditional), the predictive density behind the NLPD and the
data-space prediction against the float64 oracle, through the C ABI.

Test times cover the cases of the reference's searchsorted bridge: before the
first and after the last training time (dummy edge states), between training
times, exactly on training times (including the first and last) and on a
repeated time.  Tolerances: float64 1e-8 relative (normwise) on means and
variances, 1e-9 on the NLPD; float32 2e-4 on means and variances, 1e-4 on the
NLPD (the conditional itself runs in float64; the float32 error comes from the
smoothed states it starts from)."""
import numpy as np
import pytest

from oracle import models as OM
from oracle import ops as OO
from tests._cases import lik_pair, prior_pair, rel_err, series

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {torch.float64: (1e-8, 1e-9), torch.float32: (2e-4, 1e-4)}


def _test_times(x, seed=3, n=200):
    rng = np.random.default_rng(seed)
    span = x[-1] - x[0]
    inner = rng.uniform(x[0] - 0.1 * span, x[-1] + 0.1 * span, n)
    return np.concatenate([inner, x[[0, 1, len(x) // 2, len(x) - 1]], [x[0] - 50.0, x[-1] + 50.0]])


def _models(prior, lik, N, dtype, parallel, steps=2, lr=1.0, missing=0.0):
    import bayesnewton_gb300 as bnx
    ok, gk = prior_pair(prior)
    ol, gl = lik_pair(lik)
    x, y = series(N, lik, seed=1, missing=missing, duplicates=True)
    gm = bnx.models.MarkovVariationalGP(gk, gl, x, y, parallel=parallel, dtype=dtype)
    om = OM.MarkovGP(ok, ol, x, y)
    for _ in range(steps):
        gm.inference(lr=lr)
        om.inference(lr=lr)
    return gm, om, x, y


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("parallel", [True, False])
@pytest.mark.parametrize("prior,lik", [("m52", "gaussian"), ("sum52_32", "logit"), ("m32", "poisson"),
                                       ("m12", "probit"), ("ind52_52", "hetero_exp")])
def test_predict_matches_oracle(dtype, parallel, prior, lik):
    gm, om, x, _ = _models(prior, lik, 300, dtype, parallel, missing=0.1 if lik == "gaussian" else 0.0)
    xt = _test_times(x)
    energy0, status0 = gm.energy(), gm.status()
    m_g, v_g = gm.predict(xt)
    m_o, v_o = om.predict(xt)
    tol = TOL[dtype][0]
    assert rel_err(m_g.cpu(), m_o) < tol
    assert rel_err(v_g.cpu(), v_o) < tol
    # the step's results are left in place
    assert gm.energy() == energy0 and gm.status() == status0


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_predict_at_training_times_default(dtype):
    gm, om, x, _ = _models("m52", "gaussian", 257, dtype, True)
    m_g, v_g = gm.predict()
    m_o, v_o = om.predict(x)
    assert rel_err(m_g.cpu(), m_o) < TOL[dtype][0]
    assert rel_err(v_g.cpu(), v_o) < TOL[dtype][0]


@pytest.mark.parametrize("prior", ["m52", "sum52_32", "ind52_52"])
def test_temporal_conditional_ops(prior):
    """The ops-level operator on the oracle's own smoothed states and gains, with
    the reference's augmented time vector."""
    import bayesnewton_gb300 as bnx
    ok, gk = prior_pair(prior)
    ol, _ = lik_pair("gaussian" if prior != "ind52_52" else "hetero_exp")
    x, y = series(120, "gaussian", seed=4)
    om = OM.MarkovGP(ok, ol, x, y)
    om.inference(lr=1.0)
    _, (fm, fP) = OO.kalman_filter(om.dt, ok, om.site_mean, om.site_cov, mask=om.mask_pseudo_y)
    dts = np.concatenate([om.dt[1:], [0.0]])
    sm, sP, G = OO.rauch_tung_striebel_smoother(dts, ok, fm, fP, return_full=True)
    X_aug = np.concatenate([[-1e10], om.X[:, 0], [1e10]])
    xt = _test_times(om.X[:, 0], seed=5, n=100)
    m_o, P_o = OO.temporal_conditional(X_aug, xt, sm, sP, G, ok)
    m_g, P_g = bnx.ops.temporal_conditional(X_aug, xt, torch.as_tensor(sm).cuda(), torch.as_tensor(sP).cuda(),
                                            torch.as_tensor(G).cuda(), gk)
    assert rel_err(m_g.cpu(), m_o) < 1e-9
    assert rel_err(P_g.cpu(), P_o) < 1e-9


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("lik", ["gaussian", "logit", "probit", "poisson"])
def test_nlpd_and_predict_y(dtype, lik):
    gm, om, x, _ = _models("m52", lik, 300, dtype, True)
    xt = _test_times(x, seed=6)
    _, yt = series(xt.shape[0], lik, seed=9)
    yt[::7] = np.nan  # missing test observations are left out of the mean
    n_g = gm.negative_log_predictive_density(xt, yt)
    n_o = om.negative_log_predictive_density(xt, yt)
    assert abs(n_g - n_o) <= TOL[dtype][1] * max(1.0, abs(n_o)), (n_g, n_o)
    my_g, vy_g = gm.predict_y(xt)
    my_o, vy_o = om.predict_y(xt)
    assert rel_err(my_g.cpu(), my_o) < TOL[dtype][0]
    assert rel_err(vy_g.cpu(), vy_o) < TOL[dtype][0]


def test_predict_empty_and_errors():
    gm, _, _, _ = _models("m52", "gaussian", 50, torch.float64, True, steps=1)
    m, v = gm.predict(np.zeros(0))
    assert m.shape[0] == 0 and v.shape[0] == 0
    with pytest.raises(ValueError):
        gm.negative_log_predictive_density(np.zeros(3), np.zeros(4))


def test_predict_long_series_against_segments_of_the_oracle():
    """N = 2e5 float32: prediction through the parallel scan, checked on test times
    inside the first and last 200 training times against the oracle run on those
    windows alone.  The test times stay 50 spacings (~25 time units) away from the
    window's inner edge, where a Matern-3/2 prior with lengthscale 0.7 has
    correlation ~e^-60, so the data outside the window cannot move them."""
    import bayesnewton_gb300 as bnx
    ok, gk = prior_pair("m32")
    ol, gl = lik_pair("gaussian")
    N = 200_000
    x, y = series(N, "gaussian", seed=11, span=N * 0.5)
    gm = bnx.models.MarkovVariationalGP(gk, gl, x, y, dtype=torch.float32)
    gm.inference(lr=1.0)
    W = 200
    for sl, lo, hi in ((slice(0, W), 0, 150), (slice(N - W, N), 50, W - 1)):
        om = OM.MarkovGP(ok, ol, x[sl], y[sl])
        om.inference(lr=1.0)
        xs = x[sl]
        xt = np.random.default_rng(2).uniform(xs[lo], xs[hi], 64)
        m_g, v_g = gm.predict(xt)
        m_o, v_o = om.predict(xt)
        assert rel_err(m_g.cpu(), m_o) < 2e-4
        assert rel_err(v_g.cpu(), v_o) < 2e-4


@pytest.mark.parametrize("N", [1, 2, 3])
def test_predict_and_gradient_tiny_series(N):
    """One to three training points: the bridge's dummy edge states on both sides of a
    single point, and the gradient's head term alone."""
    import bayesnewton_gb300 as bnx
    ok, gk = prior_pair("m52")
    ol, gl = lik_pair("gaussian")
    x, y = series(N, "gaussian", seed=12)
    gm = bnx.models.MarkovVariationalGP(gk, gl, x, y, dtype=torch.float64)
    om = OM.MarkovGP(ok, ol, x, y)
    gm.inference(lr=1.0)
    om.inference(lr=1.0)
    xt = np.concatenate([x - 1.0, x, x + 0.5])
    m_g, v_g = gm.predict(xt)
    m_o, v_o = om.predict(xt)
    assert rel_err(m_g.cpu(), np.atleast_1d(m_o)) < 1e-8
    assert rel_err(v_g.cpu(), np.atleast_1d(v_o)) < 1e-8
    _, g = gm.energy_and_grad()
    g_o = OM.energy_gradient_fd(om)
    g_g = np.array(list(g.values()))
    assert np.max(np.abs(g_g - g_o)) <= 1e-6 * max(np.max(np.abs(g_o)), 1e-12)

