"""GPU parity of the batched step (many independent series in one pass) against
the float64 oracle run series by series, through the C ABI.

Tolerances as for the single-series models: float64 1e-8 relative on each
series' posterior means and variances and on each series' energy; float32 2e-4
(normwise, per series) and 1e-5 relative on the energies."""
import numpy as np
import pytest

from oracle import kernels as OK
from oracle import likelihoods as OL
from oracle import models as OM
from tests._cases import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {torch.float64: (1e-8, 1e-8), torch.float32: (2e-4, 1e-5)}
KERN = {"m12": ("Matern12", 1), "m32": ("Matern32", 2), "m52": ("Matern52", 3), "m72": ("Matern72", 4)}


def make_series(S, lmin, lmax, seed=0, liks=("gaussian", "poisson"), kern="m32", short=True):
    """Seeded series: lengths log-uniform in [lmin, lmax] (plus lengths 1, 2, 3
    when short), per-series lengthscale log-uniform in [0.5, 20], variance in
    [0.5, 2]; y from f = sin(x / ell) drawn for the series' likelihood."""
    rng = np.random.default_rng(seed)
    lens = np.exp(rng.uniform(np.log(lmin), np.log(lmax), S)).astype(int)
    if short:
        lens[:3] = [1, 2, 3]
    out = []
    for i, n in enumerate(lens):
        ell = float(np.exp(rng.uniform(np.log(0.5), np.log(20.0))))
        var = float(rng.uniform(0.5, 2.0))
        lik = liks[i % len(liks)]
        x = np.sort(rng.uniform(0.0, n / 5.0 + 1.0, n))
        f = np.sin(x / ell) + 0.3 * np.cos(x)
        if lik == "gaussian":
            noise = float(rng.uniform(0.02, 0.2))
            y = f + np.sqrt(noise) * rng.standard_normal(n)
        elif lik == "poisson":
            noise = 1.0
            y = rng.poisson(np.exp(f)).astype(float)
        else:
            noise = 1.0
            y = (rng.uniform(size=n) < 1.0 / (1.0 + np.exp(-2.0 * f))).astype(float)
        out.append(dict(kern=kern, var=var, ell=ell, lik=lik, noise=noise, x=x, y=y))
    return out


def _gpu_objs(s):
    import bayesnewton_gb300 as bnx
    k = getattr(bnx.kernels, KERN[s["kern"]][0])(s["var"], s["ell"])
    lik = {"gaussian": lambda: bnx.likelihoods.Gaussian(s["noise"]), "poisson": lambda: bnx.likelihoods.Poisson(),
           "logit": lambda: bnx.likelihoods.Bernoulli("logit")}[s["lik"]]()
    return k, lik


def _oracle_objs(s):
    k = getattr(OK, KERN[s["kern"]][0])(s["var"], s["ell"])
    lik = {"gaussian": lambda: OL.Gaussian(s["noise"]), "poisson": lambda: OL.Poisson(),
           "logit": lambda: OL.Bernoulli("logit")}[s["lik"]]()
    return k, lik


def _batch(ss, dtype, method="vi", spt=0, **kw):
    import bayesnewton_gb300 as bnx
    series = [(*_gpu_objs(s), s["x"], s["y"]) for s in ss]
    return bnx.batch.MarkovSeriesBatch(series, method=method, dtype=dtype, steps_per_thread=spt, **kw)


def _oracles(ss, method, steps, lr):
    oms = []
    for s in ss:
        ok, ol = _oracle_objs(s)
        om = OM.MarkovGP(ok, ol, s["x"], s["y"])
        for _ in range(steps):
            om.inference(lr=lr, method=method)
        oms.append(om)
    return oms


def _check_vs_oracle(b, ss, dtype, method, steps, lr, oms=None):
    tol, etol = TOL[dtype]
    if oms is None:
        oms = _oracles(ss, method, steps, lr)
    se = b.series_energy()
    for i, (s, om) in enumerate(zip(ss, oms)):
        m, v = b.series_posterior(i)
        assert rel_err(m.cpu(), om.posterior_mean.reshape(-1)) < tol, (i, s["lik"], len(s["x"]))
        assert rel_err(v.cpu(), om.posterior_variance.reshape(-1)) < tol, (i, s["lik"], len(s["x"]))
        eo = om.energy(method, 1.0)
        assert abs(se[i] - eo) <= etol * max(1.0, abs(eo)), (i, se[i], eo)
    tot = sum(om.energy(method, 1.0) for om in oms)
    assert abs(b.energy() - tot) <= etol * max(1.0, abs(tot))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("method", ["vi", "newton"])
def test_batch_mixed_likelihoods(dtype, method):
    # short chunks: most chunks and blocks straddle series boundaries
    ss = make_series(40, 5, 600, seed=1, liks=("gaussian", "poisson", "logit"))
    b = _batch(ss, dtype, method=method, spt=4)
    lr = 1.0 if method == "vi" else 0.8
    for _ in range(2):
        b.inference(lr=lr)
    _check_vs_oracle(b, ss, dtype, method, 2, lr)
    assert b.status() == 0


# Matern72 (state dim 4) has a compiled float32 layout only
@pytest.mark.parametrize("kern,dtype", [("m12", torch.float64), ("m52", torch.float64), ("m72", torch.float32)])
def test_batch_other_matern_orders(kern, dtype):
    ss = make_series(12, 3, 300, seed=2, kern=kern)
    b = _batch(ss, dtype, spt=8)
    b.inference(lr=1.0)
    _check_vs_oracle(b, ss, dtype, "vi", 1, 1.0)


def test_batch_equals_single_series_models():
    import bayesnewton_gb300 as bnx
    ss = make_series(9, 10, 400, seed=3)
    b = _batch(ss, torch.float64, spt=4)
    for _ in range(2):
        b.inference(lr=1.0)
    se = b.series_energy()
    for i, s in enumerate(ss):
        k, lik = _gpu_objs(s)
        g = bnx.models.MarkovVariationalGP(k, lik, s["x"], s["y"], dtype=torch.float64, steps_per_thread=4)
        for _ in range(2):
            g.inference(lr=1.0)
        m, v = b.series_posterior(i)
        assert rel_err(m.cpu(), g.posterior_mean.reshape(-1).cpu()) < 1e-10
        assert rel_err(v.cpu(), g.posterior_variance.reshape(-1).cpu()) < 1e-10
        assert abs(se[i] - g.energy()) <= 1e-9 * max(1.0, abs(g.energy()))


def test_batch_hyperparameter_change_and_autotune():
    ss = make_series(20, 20, 2000, seed=4)
    b = _batch(ss, torch.float64)
    oms = _oracles(ss, "vi", 1, 1.0)
    b.inference(lr=1.0)
    # a changed series hyperparameter reaches the next step (the oracle models
    # take the same change between their steps)
    b.series[5][0].lengthscale = 3.0
    oms[5].kernel.lengthscale = 3.0
    b.series[6][1].variance = 0.07
    oms[6].likelihood.variance = 0.07
    times = b.autotune(candidates=(4, 8, 16), reps=2)
    assert set(times) <= {4, 8, 16} and len(times) >= 1
    assert b.steps_per_thread in times
    b.inference(lr=1.0)
    for om in oms:
        om.inference(lr=1.0, method="vi")
    _check_vs_oracle(b, ss, torch.float64, "vi", 2, 1.0, oms=oms)


def test_batch_config_shape_against_cpu_port():
    """Many series with the shape of the 4096-series workload, scaled down
    (256 series, lengths log-uniform in [100, 5000]), float32 against the float64
    C++ port run series by series."""
    from oracle.cpu_ref import CpuRefModel
    ss = make_series(256, 100, 5000, seed=5, short=False)
    b = _batch(ss, torch.float32)
    for _ in range(2):
        b.inference(lr=1.0)
    se = b.series_energy()
    pm = b._pm[:, 0].cpu().numpy()
    errs = []
    for i, s in enumerate(ss):
        ref = CpuRefModel([("matern32", s["var"], s["ell"])], 0, s["lik"], s["x"], s["y"],
                          lik_variance=s["noise"], threads=1)
        for _ in range(2):
            ref.step(newton=True, lr=1.0)
        sl = b.series_slice(i)
        errs.append(rel_err(pm[sl], ref.pm.reshape(-1)))
        e_ref = ref.result[0]
        assert abs(se[i] - e_ref) <= 1e-5 * max(1.0, abs(e_ref)), (i, se[i], e_ref)
    assert max(errs) < 2e-4, max(errs)
