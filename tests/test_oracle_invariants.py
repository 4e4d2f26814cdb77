"""Pins the float64 oracle with the reference's own invariants, restated on seeded data.

- tests/test_vs_exact_marg_lik.py:41-59 (reference): after one lr=1 VI step with a
  Gaussian likelihood the energy equals -log N(y | 0, K + s2 I) (4 decimals there;
  far tighter here).
- tests/test_gp_vs_markovgp_reg.py:48-138 and tests/test_gp_vs_markovgp_class.py:38-124
  (reference): dense GP and Markov GP agree on the initial energy / posterior and the
  posterior after one lr=1 step (rtol 1e-4 there).
- The parallel (associative-scan) filter and smoother equal the sequential ones; the
  reference never tests this (it only runs the parallel path on a GPU backend).
- tests/test_gp_vs_markovgp_spacetime.py:86 (reference): Markov GP prediction at
  new inputs equals the dense GP's; restated here for temporal priors at test times
  before, between, on and after the training times.
"""
import numpy as np
import pytest

from oracle import kernels as K
from oracle import likelihoods as L
from oracle import models as M
from oracle import ops


def build_data(N, seed):
    # the reference's wiggly_time_series, seeded
    rng = np.random.default_rng(seed)
    x = rng.permutation(np.linspace(-25.0, 150.0, num=N) + 0.5 * rng.standard_normal(N))
    x = np.sort(x)
    y = np.cos(0.04 * x + 0.33 * np.pi) * np.sin(0.2 * x) + np.sqrt(0.15) * rng.standard_normal(N)
    return x[:, None], y


@pytest.mark.parametrize("var_f", [0.5, 1.5])
@pytest.mark.parametrize("len_f", [0.75, 2.5])
@pytest.mark.parametrize("var_y", [0.1, 0.5])
@pytest.mark.parametrize("N", [30, 60])
def test_energy_equals_exact_marginal_likelihood(var_f, len_f, var_y, N):
    x, y = build_data(N, seed=N)
    for model in (M.DenseGP(K.Matern52(var_f, len_f), L.Gaussian(var_y), x, y),
                  M.MarkovGP(K.Matern52(var_f, len_f), L.Gaussian(var_y), x, y)):
        model.inference(lr=1.0)
        Ky = K.Matern52(var_f, len_f)(x, x) + var_y * np.eye(N)
        Lc = np.linalg.cholesky(Ky)
        exact = -0.5 * y @ np.linalg.solve(Ky, y) - np.sum(np.log(np.diag(Lc))) - 0.5 * N * np.log(2 * np.pi)
        np.testing.assert_allclose(model.energy(), -exact, rtol=1e-10)


@pytest.mark.parametrize("lik", ["gaussian", "probit", "logit", "poisson"])
@pytest.mark.parametrize("parallel", [False, True])
def test_dense_vs_markov(lik, parallel):
    x, y = build_data(40, seed=7)
    if lik == "gaussian":
        mk = lambda: L.Gaussian(0.3)
    elif lik == "poisson":
        y = np.round(np.exp(y))
        mk = lambda: L.Poisson()
    else:
        y = (y > 0).astype(float)
        mk = lambda: L.Bernoulli(lik)
    gp = M.DenseGP(K.Matern52(1.5, 2.5), mk(), x, y)
    mg = M.MarkovGP(K.Matern52(1.5, 2.5), mk(), x, y, parallel=parallel)
    for m in (gp, mg):
        m.update_posterior()
    np.testing.assert_allclose(gp.energy(), mg.energy(), rtol=1e-10)
    for _ in range(2):
        for m in (gp, mg):
            m.inference(lr=1.0)
        np.testing.assert_allclose(gp.posterior_mean, mg.posterior_mean, rtol=1e-8, atol=1e-12)
        np.testing.assert_allclose(gp.posterior_variance, mg.posterior_variance, rtol=1e-8)
    np.testing.assert_allclose(gp.energy(), mg.energy(), rtol=1e-10)


@pytest.mark.parametrize("method", ["newton", "ep"])
def test_dense_vs_markov_newton_ep(method):
    x, y = build_data(40, seed=11)
    y = (y > 0).astype(float)
    gp = M.DenseGP(K.Matern32(1.2, 3.0), L.Bernoulli("logit"), x, y)
    mg = M.MarkovGP(K.Matern32(1.2, 3.0), L.Bernoulli("logit"), x, y)
    for _ in range(2):
        for m in (gp, mg):
            m.inference(lr=0.7, method=method)
    np.testing.assert_allclose(gp.posterior_mean, mg.posterior_mean, rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(gp.energy(method), mg.energy(method), rtol=1e-10)


@pytest.mark.parametrize("lik", ["gaussian", "logit", "probit", "poisson"])
def test_dense_vs_markov_posterior_linearisation(lik):
    """Posterior linearisation (inference.py:328-428): dense and Markov GP agree after
    PL steps; with a Gaussian likelihood the SLR is exact, so one lr=1 PL step gives
    the same posterior as one VI step."""
    x, y = build_data(40, seed=17)
    if lik == "gaussian":
        mk = lambda: L.Gaussian(0.3)
    elif lik == "poisson":
        y = np.round(np.exp(y))
        mk = lambda: L.Poisson()
    else:
        y = (y > 0).astype(float)
        mk = lambda: L.Bernoulli(lik)
    gp = M.DenseGP(K.Matern52(1.0, 2.0), mk(), x, y)
    mg = M.MarkovGP(K.Matern52(1.0, 2.0), mk(), x, y)
    for _ in range(3):
        for m in (gp, mg):
            m.inference(lr=1.0, method="pl")
    np.testing.assert_allclose(gp.posterior_mean, mg.posterior_mean, rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(gp.energy("pl"), mg.energy("pl"), rtol=1e-10)
    if lik == "gaussian":
        vi = M.MarkovGP(K.Matern52(1.0, 2.0), mk(), x, y)
        pl = M.MarkovGP(K.Matern52(1.0, 2.0), mk(), x, y)
        vi.inference(lr=1.0)
        pl.inference(lr=1.0, method="pl")
        np.testing.assert_allclose(pl.posterior_mean, vi.posterior_mean, rtol=1e-10, atol=1e-13)


def test_dense_vs_markov_sum_and_heteroscedastic():
    x, y = build_data(30, seed=3)
    k = lambda: K.Sum([K.Matern52(1.0, 2.0), K.Matern32(0.5, 5.0)])
    gp = M.DenseGP(k(), L.Gaussian(0.2), x, y)
    mg = M.MarkovGP(k(), L.Gaussian(0.2), x, y)
    for m in (gp, mg):
        m.inference(1.0)
    np.testing.assert_allclose(gp.posterior_mean, mg.posterior_mean, rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(gp.energy(), mg.energy(), rtol=1e-10)
    ki = lambda: K.Independent([K.Matern52(1.0, 2.0), K.Matern52(0.5, 8.0)])
    gp = M.DenseGP(ki(), L.HeteroscedasticNoise("exp"), x, y)
    mg = M.MarkovGP(ki(), L.HeteroscedasticNoise("exp"), x, y)
    for _ in range(2):
        for m in (gp, mg):
            m.inference(1.0)
    np.testing.assert_allclose(gp.posterior_mean, mg.posterior_mean, rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(gp.energy(), mg.energy(), rtol=1e-10)


@pytest.mark.parametrize("lik", ["gaussian", "logit", "poisson"])
@pytest.mark.parametrize("parallel", [False, True])
def test_markov_prediction_equals_dense_gp(lik, parallel):
    x, y = build_data(50, seed=13)
    if lik == "gaussian":
        mk = lambda: L.Gaussian(0.2)
    elif lik == "poisson":
        y = np.round(np.exp(y))
        mk = lambda: L.Poisson()
    else:
        y = (y > 0).astype(float)
        mk = lambda: L.Bernoulli("logit")
    k = lambda: K.Sum([K.Matern52(1.0, 3.0), K.Matern32(0.5, 8.0)])
    gp = M.DenseGP(k(), mk(), x, y)
    mg = M.MarkovGP(k(), mk(), x, y, parallel=parallel)
    for _ in range(2):
        for m in (gp, mg):
            m.inference(lr=1.0)
    rng = np.random.default_rng(1)
    xt = np.concatenate([rng.uniform(-40.0, 170.0, 60), x[[0, 7, 49], 0]])
    mm, vm = mg.predict(xt)
    md, vd = gp.predict(xt)
    # the bridge's 1e-8 jitter on Q_mp is the only difference
    np.testing.assert_allclose(mm, md, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(vm, vd, rtol=1e-6, atol=1e-7)
    yt = np.where(rng.uniform(size=xt.shape[0]) < 0.2, np.nan, np.interp(xt, x[:, 0], y))
    if lik != "gaussian":
        yt = np.round(yt)
    np.testing.assert_allclose(mg.negative_log_predictive_density(xt, yt),
                               gp.negative_log_predictive_density(xt, yt), rtol=1e-7)


def test_markov_prediction_two_latents_equals_dense_gp():
    x, y = build_data(30, seed=5)
    ki = lambda: K.Independent([K.Matern52(1.0, 4.0), K.Matern52(0.5, 8.0)])
    gp = M.DenseGP(ki(), L.HeteroscedasticNoise("exp"), x, y)
    mg = M.MarkovGP(ki(), L.HeteroscedasticNoise("exp"), x, y)
    for m in (gp, mg):
        m.inference(1.0)
    xt = np.random.default_rng(2).uniform(-40.0, 170.0, 40)
    mm, vm = mg.predict(xt)
    md, vd = gp.predict(xt)
    np.testing.assert_allclose(mm, md, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(vm, vd, rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("method,power", [("vi", 1.0), ("newton", 1.0), ("ep", 0.7), ("pl", 1.0)])
def test_energy_gradient_dense_equals_markov(method, power):
    """The gradient of the energy with sites and posterior held fixed (what
    objax.GradValues differentiates; tests/test_gp_vs_markovgp_reg.py:77-118 of the
    reference checks dense == Markov at the initial sites): equal for the dense and
    Markov oracles at the initial sites and after steps, for every method's energy."""
    x, y = build_data(40, seed=19)
    gp = M.DenseGP(K.Matern52(1.2, 2.5), L.Gaussian(0.3), x, y)
    mg = M.MarkovGP(K.Matern52(1.2, 2.5), L.Gaussian(0.3), x, y)
    for m in (gp, mg):
        m.update_posterior()
    np.testing.assert_allclose(M.energy_gradient_fd(gp, method=method, power=power),
                               M.energy_gradient_fd(mg, method=method, power=power), rtol=1e-6, atol=1e-8)
    for m in (gp, mg):
        m.inference(0.7, method=method, power=power)
    np.testing.assert_allclose(M.energy_gradient_fd(gp, method=method, power=power),
                               M.energy_gradient_fd(mg, method=method, power=power), rtol=1e-6, atol=1e-8)


@pytest.mark.parametrize("method", ["vi", "newton"])
def test_mean_field_equals_joint_filter_with_diagonal_sites(method):
    """The mean-field filter and smoother (ops.py:429-706) keep the latents'
    covariance block-diagonal.  With an Independent prior and diagonal site
    precisions (what ensure_diagonal_positive_precision, utils.py:89-96, gives the
    VI and Newton updates) the joint filter's covariance is block-diagonal anyway,
    so the mean-field model equals the joint one: posterior and energy after
    steps of the heteroscedastic two-latent model."""
    x, y = build_data(60, seed=23)
    ki = lambda: K.Independent([K.Matern52(1.0, 4.0), K.Matern32(0.5, 8.0)])
    mf = M.MarkovMeanFieldGP(ki(), L.HeteroscedasticNoise("exp"), x, y)
    mg = M.MarkovGP(ki(), L.HeteroscedasticNoise("exp"), x, y)
    for _ in range(3):
        for m in (mf, mg):
            m.inference(0.8, method=method)
        np.testing.assert_allclose(mf.posterior_mean, mg.posterior_mean, rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(mf.posterior_variance, mg.posterior_variance, rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(mf.energy(method), mg.energy(method), rtol=1e-12)


def test_energy_gradient_oracle_equals_exact_marginal_likelihood_gradient():
    """Pins the finite-difference gradient oracle: with a Gaussian likelihood, after
    one lr=1 VI step q is the exact posterior, so the energy's gradient at fixed q
    and sites is minus the gradient of log N(y | 0, K + s2 I), known in closed form
    as 1/2 tr((a a^T - Ky^-1) dKy), a = Ky^-1 y."""
    x, y = build_data(40, seed=29)
    var_f, len_f, var_y = 1.3, 2.2, 0.25
    mg = M.MarkovGP(K.Matern52(var_f, len_f), L.Gaussian(var_y), x, y)
    mg.inference(lr=1.0)
    g = M.energy_gradient_fd(mg)
    kmat = lambda v, l: K.Matern52(v, l)(x, x)
    Ky = kmat(var_f, len_f) + var_y * np.eye(x.shape[0])
    a = np.linalg.solve(Ky, y)
    W = np.outer(a, a) - np.linalg.inv(Ky)
    h = 1e-6 * len_f
    dKs = [kmat(var_f, len_f) / var_f, (kmat(var_f, len_f + h) - kmat(var_f, len_f - h)) / (2 * h),
           np.eye(x.shape[0])]
    exact = np.array([-0.5 * np.sum(W * d) for d in dKs])
    np.testing.assert_allclose(g, exact, rtol=1e-6, atol=1e-8)


def test_dare_fixed_point():
    """The infinite-horizon filter's Riccati recursion (ops.py:796-822) converges
    to the solution of the discrete algebraic Riccati equation."""
    from oracle import ops
    kern = K.Matern32(1.0, 1.5)
    A = kern.state_transition(0.1)
    Pinf = kern.stationary_covariance()
    Q = Pinf - A @ Pinf @ A.T
    H = kern.measurement_model()
    R = np.array([[0.2]])
    X = ops.dare(A, H, Q, R, Pinf, num_iters=400)
    S = H @ X @ H.T + R
    res = A @ (X - X @ H.T @ np.linalg.solve(S, H @ X)) @ A.T + Q - X
    assert np.max(np.abs(res)) < 1e-12 * np.max(np.abs(X))


@pytest.mark.parametrize("lik", ["gaussian", "logit"])
def test_infinite_horizon_oracle(lik):
    """The infinite-horizon restatement (ops.py:796-1068, basemodels.py:1257-1308):
    with converged Riccati recursions its posterior equals the full Markov GP's away
    from the ends of the series, and its parallel form equals the sequential one
    (both the homoscedastic and the heteroscedastic operator)."""
    rng = np.random.default_rng(3)
    N = 300
    x = np.arange(N) * 0.1
    y = np.sin(0.5 * x) + 0.3 * rng.standard_normal(N)
    mk = (lambda: L.Gaussian(0.2)) if lik == "gaussian" else (lambda: L.Bernoulli("logit"))
    if lik != "gaussian":
        y = (y > 0).astype(float)
    kern = lambda: K.Sum([K.Matern52(1.0, 2.0), K.Matern32(0.5, 0.7)])
    if lik == "gaussian":
        ih = M.InfiniteHorizonGP(kern(), mk(), x, y, dare_iters=500)
        mg = M.MarkovGP(kern(), mk(), x, y)
        ih.inference(1.0)
        mg.inference(1.0)
        np.testing.assert_allclose(ih.posterior_mean[100:200], mg.posterior_mean[100:200], atol=1e-7)
        np.testing.assert_allclose(ih.posterior_variance[100:200], mg.posterior_variance[100:200], rtol=1e-7)
    par = M.InfiniteHorizonGP(kern(), mk(), x, y, parallel=True)
    seq = M.InfiniteHorizonGP(kern(), mk(), x, y)
    for _ in range(2):
        for m in (par, seq):
            m.inference(1.0)
    np.testing.assert_allclose(par.posterior_mean, seq.posterior_mean, atol=1e-12)
    np.testing.assert_allclose(par.energy(), seq.energy(), rtol=1e-12)


@pytest.mark.parametrize("kern", [K.Matern12(1.1, 0.6), K.Matern32(0.9, 1.3), K.Matern52(1.4, 0.8),
                                  K.Matern72(0.7, 2.1)])
def test_closed_form_transition_equals_expm(kern):
    dt = np.random.default_rng(0).uniform(0.0, 3.0, 16)
    np.testing.assert_allclose(kern.state_transition(dt), K.FeedbackKernel.of(kern).state_transition(dt),
                               rtol=1e-11, atol=1e-13)


@pytest.mark.parametrize("stable", [False, True])
def test_parallel_equals_sequential_filter_smoother(stable):
    rng = np.random.default_rng(5)
    N = 257
    dt = np.concatenate([[0.0], rng.uniform(0.01, 0.5, N - 1)])
    kern = K.Sum([K.Matern52(1.0, 1.0), K.Matern32(0.5, 3.0)])
    y = rng.standard_normal([N, 1, 1])
    R = rng.uniform(0.05, 2.0, [N, 1, 1])
    mask = rng.uniform(size=[N, 1]) < 0.1
    ell_s, (fm_s, fP_s) = ops.kalman_filter(dt, kern, y, R, mask, parallel=False)
    ell_p, (fm_p, fP_p) = ops.kalman_filter(dt, kern, y, R, mask, parallel=True, stable=stable)
    np.testing.assert_allclose(ell_p, ell_s, rtol=1e-10)
    np.testing.assert_allclose(fm_p, fm_s, rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(fP_p, fP_s, rtol=1e-7, atol=1e-9)
    dts = np.concatenate([dt[1:], [0.0]])
    for full in (False, True):
        a = ops.rauch_tung_striebel_smoother(dts, kern, fm_s, fP_s, return_full=full, parallel=False)
        b = ops.rauch_tung_striebel_smoother(dts, kern, fm_s, fP_s, return_full=full, parallel=True)
        for u, v in zip(a, b):
            np.testing.assert_allclose(u, v, rtol=1e-7, atol=1e-9)


def test_cubature_matches_closed_forms():
    """The 1-D GH score-form expectation (cubature.py:198-246) against the
    closed forms the reference uses for Gaussian and Poisson."""
    g, p = L.Gaussian(0.37), L.Poisson()
    for (y, m, v) in [(0.3, -0.2, 0.5), (1.7, 0.4, 0.05), (-2.0, 1.0, 2.0)]:
        cub = L.Likelihood.ve_scalar(g, y, m, v)
        np.testing.assert_allclose(cub, g.ve_scalar(y, m, v), rtol=1e-10, atol=1e-12)
    for (y, m, v) in [(3.0, 0.5, 0.2), (0.0, -1.0, 0.1), (7.0, 1.8, 0.3)]:
        cub = L.Likelihood.ve_scalar(p, y, m, v)
        np.testing.assert_allclose(cub, p.ve_scalar(y, m, v), rtol=1e-8, atol=1e-10)


def test_spatiotemporal_oracle_equals_dense_gp_on_gridded_inputs():
    """With every time point observed at the inducing inputs (R_t = z) the
    spatial conditional is exact (B = Lzz, C = 0), so the spatio-temporal Markov
    GP is the dense GP with the separable kernel k_t k_s at those points: the
    posterior marginals and the VI energy agree before and after VI steps
    (the spatio-temporal counterpart of tests/test_gp_vs_markovgp_reg.py)."""
    from oracle import kernels as OK, likelihoods as OL, models as OM
    from oracle.spatiotemporal import SpatioTemporalKernel, STMarkovGP
    rng = np.random.default_rng(0)
    Nt, g = 10, 3
    z1 = np.linspace(0.1, 0.9, g)
    za, zb = np.meshgrid(z1, z1)
    z = np.stack([za.ravel(), zb.ravel()], 1)
    M = z.shape[0]
    X = np.sort(rng.uniform(0, 10, Nt))
    R = np.tile(z[None], [Nt, 1, 1])
    Y = rng.poisson(1.5, [Nt, M]).astype(float)
    kt, ks = OK.Matern32(1.3, 2.0), OK.Matern32(0.8, 0.4)

    class Prod:
        def __call__(self, A, B):
            return kt(A[:, :1], B[:, :1]) * ks(A[:, 1:], B[:, 1:])

    for par in (False, True):
        st = STMarkovGP(SpatioTemporalKernel(kt, ks, z), OL.Poisson(), X, R, Y, parallel=par)
        Xd = np.concatenate([np.repeat(X, M)[:, None], R.reshape(-1, 2)], 1)
        dg = OM.DenseGP(Prod(), OL.Poisson(), Xd, Y.reshape(-1, 1))
        for _ in range(2):
            st.inference(lr=1.0)
            dg.inference(lr=1.0, method="vi")
        mf, vf = st.conditional_posterior_to_data()
        np.testing.assert_allclose(mf.reshape(-1), dg.posterior_mean.reshape(-1), rtol=1e-8, atol=1e-9)
        np.testing.assert_allclose(vf.reshape(-1), dg.posterior_variance.reshape(-1), rtol=1e-8, atol=1e-9)
        np.testing.assert_allclose(st.energy(), dg.energy("vi"), rtol=1e-9)
        # prediction at new times and new spatial inputs: with the data at z the
        # residual f(t, r) - K_rz Kzz^-1 f(t, z) of the separable prior is independent
        # of the data, so the sparse conditional is exact here too
        Xt = np.concatenate([rng.uniform(-2, 12, 5), X[[0, 4]]])
        Rt = rng.uniform(0, 1, [Xt.shape[0], 4, 2])
        ms, vs = st.predict(Xt, Rt)
        Xtd = np.concatenate([np.repeat(Xt, 4)[:, None], Rt.reshape(-1, 2)], 1)
        md, vd = dg.predict(Xtd)
        np.testing.assert_allclose(ms.reshape(-1), md.reshape(-1), rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(vs.reshape(-1), vd.reshape(-1), rtol=1e-6, atol=1e-7)


def test_mlp_oracle_gradient_matches_finite_differences():
    """The learned-site network's oracle: its chain-rule gradient equals central
    finite differences of its loss (float64)."""
    from oracle import mlp
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, mlp.num_params())
    x = rng.normal(size=(17, 6))
    t = rng.normal(size=(17, 6))
    _, g = mlp.loss_grad(p, x, t)
    idx = rng.choice(p.shape[0], 60, replace=False)
    for i in idx:
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd = (mlp.loss_grad(p + e, x, t)[0] - mlp.loss_grad(p - e, x, t)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_plain_config_full_size_energy_equals_exact_marginal_likelihood():
    """The known answer of tests/test_vs_exact_marg_lik.py:41-59 at the plain
    workload's own size (N = 10,000, inputs 0.01 apart): after one lr = 1 VI step
    the oracle's energy is minus the exact log marginal likelihood from a dense
    Cholesky of K + 0.1 I."""
    from scipy.linalg import solve_triangular
    from tests._plain_config import plain_data, plain_oracle
    x, y = plain_data()
    _, _, energy = plain_oracle()
    Ky = K.Matern52(1.0, 1.0)(x[:, None], x[:, None])
    Ky[np.diag_indices_from(Ky)] += 0.1
    Lc = np.linalg.cholesky(Ky)
    del Ky
    z = solve_triangular(Lc, y, lower=True)
    exact = -0.5 * z @ z - np.sum(np.log(np.diag(Lc))) - 0.5 * x.shape[0] * np.log(2 * np.pi)
    np.testing.assert_allclose(energy, -exact, rtol=1e-10)


def test_logit_derivative_form_matches_score_form():
    """The float32 Bernoulli-logit sites take E_q[d log p / df] and
    E_q[d2 log p / df2] under the 20-point rule instead of the reference's
    score-function sums (cubature.py:198-246).  For the exact integral the two
    are equal (Stein's lemma); under the 20-point rule they agree to 1e-6
    (absolute) for posterior variances up to 2, the marginal prior variance of
    the N = 1e6 workload's Sum(Matern52, Matern32), and drift apart above it."""
    from oracle import cubature as C
    x, w = C.gauss_hermite(1, 20)
    x, w = x.reshape(-1), w.reshape(-1)

    def worst(v):
        out = 0.0
        for y in (0.0, 1.0):
            for m in np.linspace(-4.0, 4.0, 33):
                f = m + np.sqrt(v) * x
                s = 1.0 / (1.0 + np.exp(-f))
                lp = np.log(np.where(y == 1.0, s, 1.0 - s))
                _, d1s, d2s = C.variational_expectation_cubature(
                    lambda yy, ff: np.log(np.where(yy == 1.0, 1.0 / (1.0 + np.exp(-ff)), 1.0 - 1.0 / (1.0 + np.exp(-ff)))),
                    y, m, v)
                d1d, d2d = w @ (y - s), w @ (-s * (1.0 - s))
                assert np.isfinite(lp).all()
                out = max(out, abs(d1s - d1d), abs(d2s - d2d))
        return out

    for v in (0.01, 0.1, 0.5, 1.0, 2.0):
        assert worst(v) < 1e-6, v
    assert worst(4.0) > 1e-6


def test_spatiotemporal_pseudo_precision_conditioning():
    """Why the spatio-temporal update avoids the reference's pseudo variance
    R = Lam^-1 (basemodels.py:676-687) in float32: on the first 16 time points of
    the Nt = 2,000 Poisson workload, the latent pseudo precision
    Lam = B^T diag(nat2) B + 1e-12 I reaches cond > 1e6 after the second VI step;
    its float32 inverse is then off by > 1e-4 (relative), while its float64
    Cholesky factor rounded to float32 reproduces Lam to 1e-6."""
    from bench import st_workload
    from oracle.spatiotemporal import STMarkovGP, SpatioTemporalKernel
    z, X, R, Y, lt, ls = st_workload(Nt=2000)
    Nt = 16
    kern = SpatioTemporalKernel(K.Matern32(1.0, lt), K.Matern32(1.0, ls), z)
    m = STMarkovGP(kern, L.Poisson(), X[:Nt], R[:Nt], Y[:Nt])
    for _ in range(2):
        m.inference(lr=1.0)
    lam = np.einsum("nrm,nr,nrk->nmk", m.B, m.site_nat2, m.B) + 1e-12 * np.eye(m.M)
    cond = np.linalg.cond(lam)
    assert cond.max() > 1e6
    i = int(np.argmax(cond))
    R64 = np.linalg.inv(lam[i])
    R32 = np.linalg.inv(lam[i].astype(np.float32)).astype(np.float64)
    assert np.abs(R32 - R64).max() / np.abs(R64).max() > 1e-4
    Lc = np.linalg.cholesky(lam[i]).astype(np.float32).astype(np.float64)
    assert np.abs(Lc @ Lc.T - lam[i]).max() / np.abs(lam[i]).max() < 1e-6


def test_probit_derivative_form_differs_from_score_form():
    """Why probit sites keep the reference's score form in every dtype: with the
    reference's 1e-3 jitter (likelihoods.py:826-827) the 20-point rule applied
    to the derivative expectations differs from the score-function sums by more
    than 1e-2 for posterior variances up to 2 (mean in [-4, 4])."""
    from scipy.stats import norm
    from oracle import cubature as C
    x, w = C.gauss_hermite(1, 20)
    x, w = x.reshape(-1), w.reshape(-1)
    a = 1.0 - 2e-3

    def lp(y, f):
        p = norm.cdf(f) * a + 1e-3
        return np.log(np.where(y == 1.0, p, 1.0 - p))

    worst = 0.0
    for y in (0.0, 1.0):
        for m in np.linspace(-4.0, 4.0, 33):
            for v in (0.01, 0.1, 0.5, 1.0, 2.0):
                f = m + np.sqrt(v) * x
                p = norm.cdf(f) * a + 1e-3
                d1p, d2p = a * norm.pdf(f), -a * f * norm.pdf(f)
                if y == 0.0:
                    p, d1p, d2p = 1.0 - p, -d1p, -d2p
                g, h = d1p / p, (d2p * p - d1p ** 2) / p ** 2
                _, d1s, d2s = C.variational_expectation_cubature(lp, y, m, v)
                worst = max(worst, abs(w @ g - d1s), abs(w @ h - d2s))
    assert worst > 1e-2, worst
