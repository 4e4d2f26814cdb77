"""GPU parity against the committed golden fixtures (tests/golden/*.npz): the
library, through the C ABI, on each fixture's stored inputs, against the
fixture's stored float64 outputs (made by tests/golden/make_golden.py from the
oracle, and checked there against dense-GP and exact-GP values).

Tolerances, as in the other parity tests: float64 1e-9 relative (normwise) at
the ops boundary and 1e-8 on posterior means, variances and energies after the
model steps; float32 2e-5 / 5e-5 (filter / smoother), 2e-4 on posteriors and
1e-5 relative on energies; the spatio-temporal step (float32) 5e-4 and 1e-5;
prediction (float64) 1e-8 and the energy gradient (float64) 1e-6 relative to its
largest component, as in tests/test_gpu_predict.py and tests/test_gpu_grad.py;
the infinite-horizon model (float64) 1e-9 and the mean-field model (float64) 1e-8,
as in tests/test_gpu_ih.py and tests/test_gpu_models.py; the batch of series
(float64) 1e-8 per series, as in tests/test_gpu_batch.py."""
import pytest

from tests._cases import rel_err
from tests.golden.spec import library_kernel, library_likelihood, library_st_kernel
from tests.test_golden import TEMPORAL, batch_series, load

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

OPS_TOL = {torch.float64: (1e-9, 1e-9), torch.float32: (2e-5, 5e-5)}
MODEL_TOL = {torch.float64: (1e-8, 1e-8), torch.float32: (2e-4, 1e-5)}


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("parallel", [True, False])
def test_ops_fixture(dtype, parallel):
    import bayesnewton_gb300 as bnx
    g = load("ops_sum52_32_N64")
    kern = library_kernel(g["spec"]["kernel"])
    dev = torch.device("cuda", 0)
    t = lambda a: torch.as_tensor(a, dtype=dtype, device=dev)  # noqa: E731
    mask = torch.as_tensor(g["mask"], device=dev)
    ftol, stol = OPS_TOL[dtype]
    ell, (fm, fP) = bnx.ops.kalman_filter(t(g["dt"]), kern, t(g["y"]), t(g["R"]), mask, parallel=parallel)
    assert abs(ell - float(g["ell"])) <= ftol * max(1.0, abs(float(g["ell"]))) * 10
    assert rel_err(fm.cpu(), g["fm"]) < ftol
    assert rel_err(fP.cpu(), g["fP"]) < ftol
    _, (pm, pP) = bnx.ops.kalman_filter(t(g["dt"]), kern, t(g["y"]), t(g["R"]), mask, parallel=parallel,
                                        return_predict=True)
    assert rel_err(pm.cpu(), g["pm"]) < ftol
    assert rel_err(pP.cpu(), g["pP"]) < ftol
    sm, sP, G = bnx.ops.rauch_tung_striebel_smoother(t(g["dts"]), kern, t(g["fm"]), t(g["fP"]), parallel=parallel)
    assert rel_err(sm.cpu(), g["sm"]) < stol
    assert rel_err(sP.cpu(), g["sP"]) < stol
    assert rel_err(G[:-1].cpu(), g["G"][:-1]) < stol
    smf, sPf, _ = bnx.ops.rauch_tung_striebel_smoother(t(g["dts"]), kern, t(g["fm"]), t(g["fP"]), return_full=True,
                                                       parallel=parallel)
    assert rel_err(smf.cpu(), g["smf"]) < stol
    assert rel_err(sPf.cpu(), g["sPf"]) < stol


def _model(g, dtype, parallel):
    import bayesnewton_gb300 as bnx
    sp = g["spec"]
    cls = {"vi": bnx.models.MarkovVariationalGP, "newton": bnx.models.MarkovNewtonGP,
           "ep": bnx.models.MarkovExpectationPropagationGP,
           "pl": bnx.models.MarkovPosteriorLinearisationGP}[sp["method"]]
    kw = dict(power=sp["power"]) if sp["method"] == "ep" else {}
    return cls(library_kernel(sp["kernel"]), library_likelihood(sp["likelihood"]), g["x"], g["y"],
               parallel=parallel, dtype=dtype, **kw)


def _check_steps(gm, g, dtype):
    sp = g["spec"]
    tol, etol = MODEL_TOL[dtype]
    for s in range(1, sp["steps"] + 1):
        gm.inference(lr=sp["lr"])
        assert rel_err(gm.posterior_mean.cpu(), g[f"mean_{s}"]) < tol, s
        assert rel_err(gm.posterior_variance.cpu(), g[f"var_{s}"]) < tol, s
        e, ref = gm.energy(), float(g[f"energy_{s}"])
        assert abs(e - ref) <= etol * max(1.0, abs(ref)), (s, e, ref)


@pytest.mark.parametrize("parallel", [True, False])
@pytest.mark.parametrize("name", TEMPORAL)
def test_temporal_fixture_float64(name, parallel):
    g = load(name)
    _check_steps(_model(g, torch.float64, parallel), g, torch.float64)


def test_long_series_fixture_float32():
    """The fixture shaped like the long Bernoulli-logit series (Sum(Matern52,
    Matern32), 20-point Gauss-Hermite, inputs 0.01 apart), in float32 with the
    parallel scan, the form the long-series step runs in."""
    g = load("vi_sum52_32_logit_N500")
    _check_steps(_model(g, torch.float32, True), g, torch.float32)


def test_spatiotemporal_fixture():
    import bayesnewton_gb300 as bnx
    g = load("st_m32_poisson_Nt12_M9_Nr30")
    sp = g["spec"]
    gm = bnx.models.MarkovVariationalGP(library_st_kernel(sp, g["z"]), library_likelihood(sp["likelihood"]),
                                        g["X"], g["Y"], R=g["R"])
    tol, etol = 5e-4, 1e-5
    for s in range(1, sp["steps"] + 1):
        gm.inference(lr=sp["lr"])
        assert rel_err(gm.data_mean.cpu(), g[f"data_mean_{s}"]) < tol, s
        assert rel_err(gm.data_variance.cpu(), g[f"data_var_{s}"]) < tol, s
        assert rel_err(gm.posterior_mean.cpu(), g[f"mean_{s}"]) < tol, s
        assert rel_err(gm.posterior_variance.cpu(), g[f"var_{s}"]) < tol, s
        e, ref = gm.energy(), float(g[f"energy_{s}"])
        assert abs(e - ref) <= etol * max(1.0, abs(ref)), (s, e, ref)
    assert gm.status() == 0


def test_predict_fixture_float64():
    g = load("predict_sum52_32_logit_N300")
    gm = _model(g, torch.float64, True)
    for _ in range(g["spec"]["steps"]):
        gm.inference(lr=g["spec"]["lr"])
    m, v = gm.predict(g["x_test"])
    assert rel_err(m.cpu(), g["mean"]) < 1e-8
    assert rel_err(v.cpu(), g["var"]) < 1e-8


@pytest.mark.parametrize("parallel", [True, False])
def test_grad_fixture_float64(parallel):
    import numpy as np
    g = load("grad_m52_gaussian_N250")
    sp = g["spec"]
    gm = _model(g, torch.float64, parallel)
    for tag, steps in (("init", 0), ("step2", sp["steps"])):
        for _ in range(steps):
            gm.inference(lr=sp["lr"])
        e, grads = gm.energy_and_grad()
        ref = g[f"grad_{tag}"]
        got = np.array(list(grads.values()))
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) <= 1e-6 * np.max(np.abs(ref)), (tag, got, ref)
        assert abs(e - float(g[f"energy_{tag}"])) <= 1e-8 * abs(float(g[f"energy_{tag}"]))


def test_ih_fixture_float64():
    import bayesnewton_gb300 as bnx
    g = load("ih_m52_gaussian_N1000")
    sp = g["spec"]
    gm = bnx.infinite_horizon.InfiniteHorizonVariationalGP(library_kernel(sp["kernel"]),
                                                           library_likelihood(sp["likelihood"]), g["x"], g["y"],
                                                           dtype=torch.float64)
    for s in range(1, sp["steps"] + 1):
        gm.inference(lr=sp["lr"])
        assert rel_err(gm.posterior_mean.cpu(), g[f"mean_{s}"]) < 1e-9, s
        assert rel_err(gm.posterior_variance.cpu(), g[f"var_{s}"]) < 1e-9, s
        e, ref = gm.energy(), float(g[f"energy_{s}"])
        assert abs(e - ref) <= 1e-9 * max(1.0, abs(ref)), (s, e, ref)


def test_meanfield_fixture_float64():
    import bayesnewton_gb300 as bnx
    g = load("meanfield_vi_hetero_N150")
    sp = g["spec"]
    gm = bnx.models.MarkovVariationalMeanFieldGP(library_kernel(sp["kernel"]), library_likelihood(sp["likelihood"]),
                                                 g["x"], g["y"], dtype=torch.float64)
    _check_steps(gm, g, torch.float64)


def test_batch_fixture_float64():
    import bayesnewton_gb300 as bnx
    g = load("batch_m32_mixed_S6")
    sp = g["spec"]
    parts = batch_series(g)
    series = [(library_kernel(ks), library_likelihood(ls), x, y) for ks, ls, x, y, _ in parts]
    b = bnx.batch.MarkovSeriesBatch(series, dtype=torch.float64)
    for _ in range(sp["steps"]):
        b.inference(lr=sp["lr"])
    se = b.series_energy()
    for i, (_, _, _, _, sl) in enumerate(parts):
        m, v = b.series_posterior(i)
        assert rel_err(m.cpu(), g["mean"][sl]) < 1e-8, i
        assert rel_err(v.cpu(), g["var"][sl]) < 1e-8, i
        assert abs(se[i] - g["energy"][i]) <= 1e-8 * max(1.0, abs(g["energy"][i])), (i, se[i], g["energy"][i])
