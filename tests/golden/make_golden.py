"""Generate the golden fixtures under tests/golden/ (run from the repository root:
``python tests/golden/make_golden.py``).

The reference (BayesNewton 1.3.4 on jax 0.4.14 / objax) cannot be imported in
this environment, so the golden outputs come from the float64 oracle
(``oracle/``), which the invariant tests pin to the reference's own known answers
(dense GP == Markov GP, energy == minus the exact log marginal likelihood).  Each
fixture also carries values computed WITHOUT the oracle's Kalman code: the dense
GP of ``oracle.models.DenseGP`` on every temporal case, and, on the Gaussian case,
the exact GP posterior and log marginal likelihood written out below with plain
dense numpy algebra.

Every fixture holds its seeded inputs, so the tests need neither this script nor
a random generator.  The cases follow the shapes and value laws of the workloads
the library is built for, shrunk to sizes a dense float64 solve finishes in
milliseconds:

- ops_sum52_32_N64        filter / smoother at the ops boundary
                          (ops.py:256-285, :357-380) on random dt, y, R, mask;
- vi_m52_gaussian_N400    Matern52, Gaussian noise 0.1, y = sin x + 0.3 cos 3x + noise,
                          x ~ U[0, 4] (the spacing of 1e4 points on [0, 100]);
- vi_sum52_32_logit_N500  Sum(Matern52, Matern32), Bernoulli-logit, 20-point GH,
                          y ~ Bern(sigmoid(2 sin(x / 5))), x ~ U[0, 5];
- vi_m32_poisson_N300     Matern32, Poisson (exp link), f drawn from the prior;
- vi_hetero_exp_N150      two Matern52 latents, heteroscedastic noise (exp link),
                          20 x 20 GH, y = f1 + exp(f2) eps with f from the prior;
- newton_m32_logit_N200, ep_m32_logit_N200 (power 0.7), pl_m52_probit_N200;
- st_m32_poisson_Nt12_M9_Nr30  spatio-temporal VI, Matern32 x Matern32, 3 x 3
                          inducing grid, Poisson counts with f from the separable prior;
- predict_sum52_32_logit_N300  prediction (basemodels.py:766-816) after two VI steps at
                          test times before, between, on and after the training times;
- grad_m52_gaussian_N250  the hyperparameter gradient of the VI energy with sites and
                          posterior held fixed (objax.GradValues(model.energy)), at the
                          initial sites and after two steps, by central differences;
- ih_m52_gaussian_N1000   the infinite-horizon VI model (basemodels.py:1257-1308,
                          ops.py:796-1068) on equidistant times, three lr = 0.9 steps;
- meanfield_vi_hetero_N150  the mean-field VI model (basemodels.py:1158-1175, ops.py:429-706),
                          two latents, heteroscedastic noise, two lr = 0.8 steps, with the
                          joint model's values (equal: VI keeps the sites diagonal);
- batch_m32_mixed_S6      six independent Matern32 series of lengths 1 to 800 with their own
                          hyperparameters and Gaussian / Poisson / Bernoulli likelihoods, two
                          lr = 1 VI steps, each series' oracle values (concatenated, with offsets).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from tests.golden.spec import oracle_kernel, oracle_likelihood  # noqa: E402

LOG2PI = np.log(2.0 * np.pi)


def _matern52_dense(x, var, ell):
    r = np.abs(x[:, None] - x[None, :]) / ell
    s5 = np.sqrt(5.0) * r
    return var * (1.0 + s5 + 5.0 / 3.0 * r * r) * np.exp(-s5)


def _exact_gaussian(x, y, var, ell, noise):
    """Exact GP regression with a Matern52 prior, by a dense Cholesky."""
    K = _matern52_dense(x, var, ell)
    Ky = K + noise * np.eye(x.shape[0])
    L = np.linalg.cholesky(Ky)
    a = np.linalg.solve(L.T, np.linalg.solve(L, y))
    lml = -0.5 * y @ a - np.sum(np.log(np.diag(L))) - 0.5 * x.shape[0] * LOG2PI
    V = np.linalg.solve(L, K)
    return K @ a, np.diag(K) - np.sum(V * V, axis=0), float(lml)


def _prior_sample(x, kern, rng, jitter=1e-9):
    K = kern(x[:, None], x[:, None])
    return np.linalg.cholesky(K + jitter * np.eye(x.shape[0])) @ rng.standard_normal(x.shape[0])


def _save(name, spec, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, spec=np.array(json.dumps(spec)), **arrays)
    print(f"{path}: {os.path.getsize(path)} bytes")


def _temporal(name, spec, x, y):
    from oracle import models as OM
    out = dict(x=x, y=y)
    k = lambda: oracle_kernel(spec["kernel"])  # noqa: E731
    li = lambda: oracle_likelihood(spec["likelihood"])  # noqa: E731
    om = OM.MarkovGP(k(), li(), x, y)
    dm = OM.DenseGP(k(), li(), x, y)
    meth, lr, power = spec["method"], spec["lr"], spec.get("power", 1.0)
    for s in range(1, spec["steps"] + 1):
        for m in (om, dm):
            m.inference(lr=lr, method=meth, power=power)
        out[f"mean_{s}"] = om.posterior_mean
        out[f"var_{s}"] = om.posterior_variance
        out[f"energy_{s}"] = np.float64(om.energy(meth, power))
        out[f"dense_mean_{s}"] = dm.posterior_mean
        out[f"dense_var_{s}"] = dm.posterior_variance
        out[f"dense_energy_{s}"] = np.float64(dm.energy(meth, power))
    return out


def make_ops():
    from oracle import ops as OO
    spec = dict(kind="ops", kernel=["Sum", ["Matern52", 1.0, 1.5], ["Matern32", 0.5, 4.0]])
    kern = oracle_kernel(spec["kernel"])
    rng = np.random.default_rng(101)
    N, P = 64, 1
    dt = np.concatenate([[0.0], rng.uniform(0.01, 0.3, N - 1)])
    y = rng.standard_normal([N, P, 1])
    R = rng.uniform(0.05, 1.0, [N, P, P])
    mask = rng.uniform(size=[N, P]) < 0.1
    ell, (fm, fP) = OO.kalman_filter(dt, kern, y, R, mask)
    _, (pm, pP) = OO.kalman_filter(dt, kern, y, R, mask, return_predict=True)
    dts = np.concatenate([dt[1:], [0.0]])
    sm, sP, G = OO.rauch_tung_striebel_smoother(dts, kern, fm, fP)
    smf, sPf, _ = OO.rauch_tung_striebel_smoother(dts, kern, fm, fP, return_full=True)
    _save("ops_sum52_32_N64", spec, dt=dt, y=y, R=R, mask=mask, ell=np.float64(ell), fm=fm, fP=fP, pm=pm,
          pP=pP, dts=dts, sm=sm, sP=sP, G=G, smf=smf, sPf=sPf)


def make_gaussian():
    spec = dict(kind="temporal", kernel=["Matern52", 1.0, 1.0], likelihood=["Gaussian", 0.1], method="vi",
                lr=1.0, steps=1)
    rng = np.random.default_rng(1)
    N = 400
    x = np.sort(rng.uniform(0.0, 4.0, N))
    y = np.sin(x) + 0.3 * np.cos(3.0 * x) + np.sqrt(0.1) * rng.standard_normal(N)
    out = _temporal("vi_m52_gaussian_N400", spec, x, y)
    em, ev, lml = _exact_gaussian(x, y, 1.0, 1.0, 0.1)
    _save("vi_m52_gaussian_N400", spec, exact_mean=em, exact_var=ev, exact_lml=np.float64(lml), **out)


def make_logit():
    spec = dict(kind="temporal", kernel=["Sum", ["Matern52", 1.0, 1.0], ["Matern32", 1.0, 1.0]],
                likelihood=["Bernoulli", "logit"], method="vi", lr=1.0, steps=2)
    rng = np.random.default_rng(2)
    N = 500
    x = np.sort(rng.uniform(0.0, 5.0, N))
    y = (rng.uniform(size=N) < 1.0 / (1.0 + np.exp(-2.0 * np.sin(x / 5.0)))).astype(float)
    _save("vi_sum52_32_logit_N500", spec, **_temporal("vi_sum52_32_logit_N500", spec, x, y))


def make_poisson():
    spec = dict(kind="temporal", kernel=["Matern32", 1.0, 4.0], likelihood=["Poisson"], method="vi", lr=1.0,
                steps=2)
    rng = np.random.default_rng(3)
    N = 300
    x = np.sort(rng.uniform(0.0, float(N), N))
    f = _prior_sample(x, oracle_kernel(spec["kernel"]), rng)
    y = rng.poisson(np.exp(f)).astype(float)
    _save("vi_m32_poisson_N300", spec, f=f, **_temporal("vi_m32_poisson_N300", spec, x, y))


def make_hetero():
    spec = dict(kind="temporal", kernel=["Independent", ["Matern52", 1.0, 2.0], ["Matern52", 0.5, 5.0]],
                likelihood=["HeteroscedasticNoise", "exp"], method="vi", lr=1.0, steps=2)
    rng = np.random.default_rng(4)
    N = 150
    x = np.sort(rng.uniform(0.0, 15.0, N))
    parts = spec["kernel"][1:]
    f1 = _prior_sample(x, oracle_kernel(parts[0]), rng)
    f2 = _prior_sample(x, oracle_kernel(parts[1]), rng)
    y = f1 + np.exp(f2) * rng.standard_normal(N)
    _save("vi_hetero_exp_N150", spec, **_temporal("vi_hetero_exp_N150", spec, x, y))


def make_methods():
    rng = np.random.default_rng(5)
    N = 200
    x = np.sort(rng.uniform(0.0, 20.0, N))
    f = np.sin(x / 3.0) + 0.3 * np.cos(x)
    y = (rng.uniform(size=N) < 1.0 / (1.0 + np.exp(-2.0 * f))).astype(float)
    for meth, power in (("newton", 1.0), ("ep", 0.7)):
        spec = dict(kind="temporal", kernel=["Matern32", 1.2, 3.0], likelihood=["Bernoulli", "logit"],
                    method=meth, lr=0.8, power=power, steps=2)
        name = f"{meth}_m32_logit_N200"
        _save(name, spec, **_temporal(name, spec, x, y))
    spec = dict(kind="temporal", kernel=["Matern52", 1.0, 2.0], likelihood=["Bernoulli", "probit"], method="pl",
                lr=0.8, steps=2)
    _save("pl_m52_probit_N200", spec, **_temporal("pl_m52_probit_N200", spec, x, y))


def make_st():
    from oracle.spatiotemporal import STMarkovGP
    from tests.golden.spec import oracle_st_kernel
    spec = dict(kind="st", temporal=["Matern32", 1.3, 3.0], spatial=["Matern32", 0.9, 0.4],
                likelihood=["Poisson"], lr=1.0, steps=2)
    rng = np.random.default_rng(6)
    Nt, g, Nr = 12, 3, 30
    z1 = np.linspace(0.1, 0.9, g)
    za, zb = np.meshgrid(z1, z1)
    z = np.stack([za.ravel(), zb.ravel()], 1)
    X = np.sort(rng.uniform(0.0, Nt / 2.0, Nt))
    R = rng.uniform(0.0, 1.0, [Nt, Nr, 2])
    # f from the separable prior k_t(t, t') k_s(r, r') at all Nt * Nr inputs
    kt, ks = oracle_kernel(spec["temporal"]), oracle_kernel(spec["spatial"])
    T = np.repeat(X, Nr)[:, None]
    Rf = R.reshape(-1, 2)
    K = kt(T, T) * ks(Rf, Rf)
    f = (np.linalg.cholesky(K + 1e-9 * np.eye(K.shape[0])) @ rng.standard_normal(K.shape[0])).reshape(Nt, Nr)
    Y = rng.poisson(np.exp(f)).astype(float)
    om = STMarkovGP(oracle_st_kernel(spec, z), oracle_likelihood(spec["likelihood"]), X, R, Y)
    out = dict(z=z, X=X, R=R, Y=Y, f=f)
    for s in range(1, spec["steps"] + 1):
        om.inference(lr=spec["lr"])
        mf, vf = om.conditional_posterior_to_data()
        out[f"data_mean_{s}"], out[f"data_var_{s}"] = mf, vf
        out[f"mean_{s}"], out[f"var_{s}"] = om.posterior_mean, om.posterior_variance
        out[f"energy_{s}"] = np.float64(om.energy())
    _save("st_m32_poisson_Nt12_M9_Nr30", spec, **out)


def make_predict():
    from oracle import models as OM
    spec = dict(kind="predict", kernel=["Sum", ["Matern52", 1.0, 1.5], ["Matern32", 0.5, 4.0]],
                likelihood=["Bernoulli", "logit"], method="vi", lr=1.0, steps=2)
    rng = np.random.default_rng(7)
    N = 300
    x = np.sort(rng.uniform(0.0, 30.0, N))
    x[N // 2] = x[N // 2 - 1]  # a repeated training time
    y = (rng.uniform(size=N) < 1.0 / (1.0 + np.exp(-2.0 * np.sin(x / 3.0)))).astype(float)
    xt = np.concatenate([rng.uniform(-3.0, 33.0, 120), x[[0, 1, N // 2, N - 1]], [x[0] - 50.0, x[-1] + 50.0]])
    k = lambda: oracle_kernel(spec["kernel"])  # noqa: E731
    li = lambda: oracle_likelihood(spec["likelihood"])  # noqa: E731
    om, dm = OM.MarkovGP(k(), li(), x, y), OM.DenseGP(k(), li(), x, y)
    for _ in range(spec["steps"]):
        om.inference(lr=spec["lr"])
        dm.inference(lr=spec["lr"])
    m, v = om.predict(xt)
    dmean, dvar = dm.predict(xt)
    _save("predict_sum52_32_logit_N300", spec, x=x, y=y, x_test=xt, mean=m, var=v, dense_mean=dmean,
          dense_var=dvar)


def make_grad():
    from oracle import models as OM
    spec = dict(kind="grad", kernel=["Matern52", 1.2, 2.5], likelihood=["Gaussian", 0.3], method="vi", lr=0.8,
                steps=2)
    rng = np.random.default_rng(8)
    N = 250
    x = np.sort(rng.uniform(0.0, 25.0, N))
    y = np.sin(x / 3.0) + 0.3 * np.cos(x) + np.sqrt(0.3) * rng.standard_normal(N)
    k = lambda: oracle_kernel(spec["kernel"])  # noqa: E731
    li = lambda: oracle_likelihood(spec["likelihood"])  # noqa: E731
    out = dict(x=x, y=y)
    for tag, steps in (("init", 0), ("step2", spec["steps"])):
        om, dm = OM.MarkovGP(k(), li(), x, y), OM.DenseGP(k(), li(), x, y)
        for m in (om, dm):
            m.update_posterior()
            for _ in range(steps):
                m.inference(lr=spec["lr"])
        out[f"energy_{tag}"] = np.float64(om.energy())
        out[f"grad_{tag}"] = OM.energy_gradient_fd(om)
        out[f"dense_grad_{tag}"] = OM.energy_gradient_fd(dm)
    _save("grad_m52_gaussian_N250", spec, **out)


def make_ih():
    from oracle import models as OM
    spec = dict(kind="ih", kernel=["Matern52", 1.0, 1.0], likelihood=["Gaussian", 0.1], method="vi", lr=0.9,
                steps=3)
    rng = np.random.default_rng(9)
    N = 1000
    x = np.arange(N) * 0.1 + 3.0
    y = np.sin(x / 3.0) + 0.3 * np.cos(x) + np.sqrt(0.1) * rng.standard_normal(N)
    om = OM.InfiniteHorizonGP(oracle_kernel(spec["kernel"]), oracle_likelihood(spec["likelihood"]), x, y)
    out = dict(x=x, y=y)
    for s_ in range(1, spec["steps"] + 1):
        om.inference(lr=spec["lr"], method="vi")
        out[f"mean_{s_}"], out[f"var_{s_}"] = om.posterior_mean, om.posterior_variance
        out[f"energy_{s_}"] = np.float64(om.energy("vi"))
    _save("ih_m52_gaussian_N1000", spec, **out)


def make_meanfield():
    from oracle import models as OM
    spec = dict(kind="meanfield", kernel=["Independent", ["Matern52", 1.0, 2.0], ["Matern52", 0.5, 5.0]],
                likelihood=["HeteroscedasticNoise", "exp"], method="vi", lr=0.8, steps=2)
    rng = np.random.default_rng(10)
    N = 150
    x = np.sort(rng.uniform(0.0, 15.0, N))
    parts = spec["kernel"][1:]
    f1 = _prior_sample(x, oracle_kernel(parts[0]), rng)
    f2 = _prior_sample(x, oracle_kernel(parts[1]), rng)
    y = f1 + np.exp(f2) * rng.standard_normal(N)
    k = lambda: oracle_kernel(spec["kernel"])  # noqa: E731
    li = lambda: oracle_likelihood(spec["likelihood"])  # noqa: E731
    mf, jm = OM.MarkovMeanFieldGP(k(), li(), x, y), OM.MarkovGP(k(), li(), x, y)
    out = dict(x=x, y=y)
    for s_ in range(1, spec["steps"] + 1):
        for m in (mf, jm):
            m.inference(lr=spec["lr"], method="vi")
        out[f"mean_{s_}"], out[f"var_{s_}"] = mf.posterior_mean, mf.posterior_variance
        out[f"energy_{s_}"] = np.float64(mf.energy("vi"))
        out[f"joint_mean_{s_}"], out[f"joint_var_{s_}"] = jm.posterior_mean, jm.posterior_variance
        out[f"joint_energy_{s_}"] = np.float64(jm.energy("vi"))
    _save("meanfield_vi_hetero_N150", spec, **out)


def make_batch():
    from oracle import models as OM
    rng = np.random.default_rng(11)
    lens = [1, 2, 50, 200, 400, 800]
    liks = [["Gaussian", 0.05], ["Poisson"], ["Bernoulli", "logit"], ["Gaussian", 0.2], ["Poisson"],
            ["Bernoulli", "logit"]]
    spec = dict(kind="batch", family="Matern32", likelihoods=liks, method="vi", lr=1.0, steps=2)
    xs, ys, var, ell, ms, vs, es = [], [], [], [], [], [], []
    for n, lk in zip(lens, liks):
        v, l = float(rng.uniform(0.5, 2.0)), float(np.exp(rng.uniform(np.log(0.5), np.log(20.0))))
        x = np.sort(rng.uniform(0.0, n / 5.0 + 1.0, n))
        f = _prior_sample(x, oracle_kernel(["Matern32", v, l]), rng) if n > 1 else rng.standard_normal(1) * v ** 0.5
        if lk[0] == "Gaussian":
            y = f + np.sqrt(lk[1]) * rng.standard_normal(n)
        elif lk[0] == "Poisson":
            y = rng.poisson(np.exp(f)).astype(float)
        else:
            y = (rng.uniform(size=n) < 1.0 / (1.0 + np.exp(-f))).astype(float)
        om = OM.MarkovGP(oracle_kernel(["Matern32", v, l]), oracle_likelihood(lk), x, y)
        for _ in range(spec["steps"]):
            om.inference(lr=spec["lr"])
        xs.append(x), ys.append(y), var.append(v), ell.append(l)
        ms.append(om.posterior_mean.reshape(-1)), vs.append(om.posterior_variance.reshape(-1))
        es.append(om.energy())
    _save("batch_m32_mixed_S6", spec, offsets=np.concatenate([[0], np.cumsum(lens)]), x=np.concatenate(xs),
          y=np.concatenate(ys), variance=np.array(var), lengthscale=np.array(ell), mean=np.concatenate(ms),
          var=np.concatenate(vs), energy=np.array(es))


if __name__ == "__main__":
    make_ops()
    make_gaussian()
    make_logit()
    make_poisson()
    make_hetero()
    make_methods()
    make_st()
    make_predict()
    make_grad()
    make_ih()
    make_meanfield()
    make_batch()
