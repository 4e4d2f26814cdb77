"""The committed golden fixtures (tests/golden/*.npz, written by
tests/golden/make_golden.py) against the float64 oracle and against the values
in them that do not come from the oracle's Kalman code.

- The oracle, run again on each fixture's stored inputs, reproduces the stored
  outputs to 1e-9 relative (normwise), sequentially and as the parallel scan
  with the (I + C1 J2)^-1 combine the library uses.  The reference's own combine
  (ops.py:203-219) inverts C1 and breaks down on the fixtures whose inputs are
  as dense as the long-series workloads' (dt = 0.01 at lengthscale 1), which
  test_reference_parallel_combine_breaks_down_at_dense_inputs records.
- The stored Markov-GP posterior and energy equal the stored dense-GP ones
  (oracle.models.DenseGP, no state-space algebra) to 1e-8 / 1e-9 relative, the
  invariant of bayesnewton's tests/test_gp_vs_markovgp_reg.py:48-138 and
  tests/test_gp_vs_markovgp_class.py:38-124.
- On the Gaussian fixture the energy after one lr = 1 VI step is minus the exact
  log marginal likelihood and the posterior is the exact GP posterior, both
  computed by the fixture script with plain dense algebra (the known answer of
  bayesnewton's tests/test_vs_exact_marg_lik.py:41-59), to 1e-10 / 1e-8."""
import glob
import json
import os

import numpy as np
import pytest

from tests._cases import rel_err
from tests.golden.spec import oracle_kernel, oracle_likelihood, oracle_st_kernel

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["ops_sum52_32_N64", "vi_m52_gaussian_N400", "vi_sum52_32_logit_N500", "vi_m32_poisson_N300",
         "vi_hetero_exp_N150", "newton_m32_logit_N200", "ep_m32_logit_N200", "pl_m52_probit_N200",
         "st_m32_poisson_Nt12_M9_Nr30", "predict_sum52_32_logit_N300", "grad_m52_gaussian_N250",
         "ih_m52_gaussian_N1000", "meanfield_vi_hetero_N150", "batch_m32_mixed_S6"]
TEMPORAL = [n for n in NAMES
            if not n.startswith(("ops_", "st_", "predict_", "grad_", "ih_", "meanfield_", "batch_"))]


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False) as z:
        d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    return d


def test_every_fixture_is_listed():
    found = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    assert found == sorted(NAMES)


def test_ops_fixture_reproduced_by_oracle():
    from oracle import ops as OO
    g = load("ops_sum52_32_N64")
    kern = oracle_kernel(g["spec"]["kernel"])
    for parallel in (False, True):
        ell, (fm, fP) = OO.kalman_filter(g["dt"], kern, g["y"], g["R"], g["mask"], parallel=parallel)
        assert abs(ell - g["ell"]) <= 1e-9 * abs(g["ell"])
        assert rel_err(fm, g["fm"]) < 1e-9 and rel_err(fP, g["fP"]) < 1e-9
        _, (pm, pP) = OO.kalman_filter(g["dt"], kern, g["y"], g["R"], g["mask"], parallel=parallel,
                                       return_predict=True)
        assert rel_err(pm, g["pm"]) < 1e-9 and rel_err(pP, g["pP"]) < 1e-9
        sm, sP, G = OO.rauch_tung_striebel_smoother(g["dts"], kern, g["fm"], g["fP"], parallel=parallel)
        assert rel_err(sm, g["sm"]) < 1e-9 and rel_err(sP, g["sP"]) < 1e-9
        assert rel_err(G[:-1], g["G"][:-1]) < 1e-9
        smf, sPf, _ = OO.rauch_tung_striebel_smoother(g["dts"], kern, g["fm"], g["fP"], return_full=True,
                                                      parallel=parallel)
        assert rel_err(smf, g["smf"]) < 1e-9 and rel_err(sPf, g["sPf"]) < 1e-9


@pytest.mark.parametrize("parallel", [False, True])
@pytest.mark.parametrize("name", TEMPORAL)
def test_temporal_fixture_reproduced_by_oracle(name, parallel):
    from oracle import models as OM
    g = load(name)
    sp = g["spec"]
    m = OM.MarkovGP(oracle_kernel(sp["kernel"]), oracle_likelihood(sp["likelihood"]), g["x"], g["y"],
                    parallel=parallel, stable=parallel)
    power = sp.get("power", 1.0)
    for s in range(1, sp["steps"] + 1):
        m.inference(lr=sp["lr"], method=sp["method"], power=power)
        assert rel_err(m.posterior_mean, g[f"mean_{s}"]) < 1e-9
        assert rel_err(m.posterior_variance, g[f"var_{s}"]) < 1e-9
        e = m.energy(sp["method"], power)
        assert abs(e - g[f"energy_{s}"]) <= 1e-9 * max(1.0, abs(g[f"energy_{s}"]))


@pytest.mark.parametrize("name", TEMPORAL)
def test_temporal_fixture_markov_equals_dense(name):
    g = load(name)
    for s in range(1, g["spec"]["steps"] + 1):
        assert rel_err(g[f"mean_{s}"], g[f"dense_mean_{s}"]) < 1e-8
        assert rel_err(g[f"var_{s}"], g[f"dense_var_{s}"]) < 1e-8
        assert abs(g[f"energy_{s}"] - g[f"dense_energy_{s}"]) <= 1e-9 * max(1.0, abs(g[f"dense_energy_{s}"]))


def test_gaussian_fixture_equals_exact_gp():
    g = load("vi_m52_gaussian_N400")
    assert abs(g["energy_1"] + g["exact_lml"]) <= 1e-10 * abs(g["exact_lml"])
    assert rel_err(g["mean_1"].reshape(-1), g["exact_mean"]) < 1e-8
    assert rel_err(g["var_1"].reshape(-1), g["exact_var"]) < 1e-8


def test_st_fixture_reproduced_by_oracle():
    from oracle.spatiotemporal import STMarkovGP
    g = load("st_m32_poisson_Nt12_M9_Nr30")
    sp = g["spec"]
    for parallel in (False, True):
        m = STMarkovGP(oracle_st_kernel(sp, g["z"]), oracle_likelihood(sp["likelihood"]), g["X"], g["R"], g["Y"],
                       parallel=parallel)
        for s in range(1, sp["steps"] + 1):
            m.inference(lr=sp["lr"])
            mf, vf = m.conditional_posterior_to_data()
            assert rel_err(mf, g[f"data_mean_{s}"]) < 1e-9 and rel_err(vf, g[f"data_var_{s}"]) < 1e-9
            assert rel_err(m.posterior_mean, g[f"mean_{s}"]) < 1e-9
            assert rel_err(m.posterior_variance, g[f"var_{s}"]) < 1e-9
            assert abs(m.energy() - g[f"energy_{s}"]) <= 1e-9 * max(1.0, abs(g[f"energy_{s}"]))


def test_fixture_inputs_follow_their_laws():
    """Sorted inputs and the likelihoods' supports: counts are non-negative
    integers, binary labels are 0 / 1."""
    for name in TEMPORAL:
        g = load(name)
        assert np.all(np.diff(g["x"]) >= 0)
        lik = g["spec"]["likelihood"][0]
        if lik == "Poisson":
            assert np.all(g["y"] >= 0) and np.all(g["y"] == np.round(g["y"]))
        if lik == "Bernoulli":
            assert set(np.unique(g["y"])) <= {0.0, 1.0}
    st = load("st_m32_poisson_Nt12_M9_Nr30")
    assert np.all(np.diff(st["X"]) >= 0) and np.all(st["Y"] >= 0)


@pytest.mark.parametrize("name", ["vi_m52_gaussian_N400", "vi_sum52_32_logit_N500"])
def test_reference_parallel_combine_breaks_down_at_dense_inputs(name):
    """ops.py:203-219 combines filter elements through inv(C1), C1 = Q - K H Q.
    With inputs 0.01 apart at lengthscale 1 the smallest eigenvalue of the
    Matern52 process noise Q falls as dt^5, C1 is smaller still, and in float64
    rounding C1 loses positive definiteness: the Cholesky inside inv fails (the
    reference's jax cho_factor returns NaN there instead of raising).
    The combine written with (I + C1 J2)^-1 has no inverse of C1 and reproduces
    the sequential filter on the same inputs (the test above)."""
    from oracle import models as OM
    g = load(name)
    sp = g["spec"]
    m = OM.MarkovGP(oracle_kernel(sp["kernel"]), oracle_likelihood(sp["likelihood"]), g["x"], g["y"],
                    parallel=True, stable=False)
    with pytest.raises(np.linalg.LinAlgError):
        m.inference(lr=sp["lr"], method=sp["method"])


def test_specs_build_library_objects():
    """Each fixture's specification builds the library's kernel and likelihood
    (host-side objects, no device work) with the oracle's state dimension."""
    from tests.golden.spec import library_kernel, library_likelihood, library_st_kernel
    for name in NAMES:
        g = load(name)
        sp = g["spec"]
        if sp["kind"] == "st":
            assert library_st_kernel(sp, g["z"]).state_dim == 2 * oracle_st_kernel(sp, g["z"]).M
        elif sp["kind"] == "batch":
            for ks, ls, _, _, _ in batch_series(g):
                assert library_kernel(ks).state_dim == oracle_kernel(ks).state_dim
                assert type(library_likelihood(ls)).__name__ == ls[0]
        else:
            assert library_kernel(sp["kernel"]).state_dim == oracle_kernel(sp["kernel"]).state_dim
        if "likelihood" in sp:
            assert type(library_likelihood(sp["likelihood"])).__name__ == sp["likelihood"][0]


def test_predict_fixture_reproduced_by_oracle_and_dense_gp():
    """Prediction after two VI steps (basemodels.py:766-816) at test times before,
    between, on (incl. a repeated time) and after the training times: the oracle
    reproduces the fixture (1e-9) and the stored Markov prediction equals the
    dense GP's (5e-8: the Markov bridge adds the reference's 1e-8 jitter to
    Q_mp, utils.py:123-138)."""
    from oracle import models as OM
    g = load("predict_sum52_32_logit_N300")
    sp = g["spec"]
    m = OM.MarkovGP(oracle_kernel(sp["kernel"]), oracle_likelihood(sp["likelihood"]), g["x"], g["y"])
    for _ in range(sp["steps"]):
        m.inference(lr=sp["lr"])
    mean, var = m.predict(g["x_test"])
    assert rel_err(mean, g["mean"]) < 1e-9 and rel_err(var, g["var"]) < 1e-9
    assert rel_err(g["mean"], g["dense_mean"]) < 5e-8
    assert rel_err(g["var"], g["dense_var"]) < 5e-8


def test_grad_fixture_reproduced_by_oracle_and_dense_gp():
    """Energy gradient with sites and posterior held fixed, at the initial sites
    and after two lr = 0.8 steps: the oracle's central differences reproduce the
    fixture (1e-9) and equal the dense GP's (1e-8, relative to the largest
    component), the check of bayesnewton's tests/test_gp_vs_markovgp_reg.py:77-118."""
    from oracle import models as OM
    g = load("grad_m52_gaussian_N250")
    sp = g["spec"]
    for tag, steps in (("init", 0), ("step2", sp["steps"])):
        m = OM.MarkovGP(oracle_kernel(sp["kernel"]), oracle_likelihood(sp["likelihood"]), g["x"], g["y"])
        m.update_posterior()
        for _ in range(steps):
            m.inference(lr=sp["lr"])
        assert abs(m.energy() - g[f"energy_{tag}"]) <= 1e-9 * abs(g[f"energy_{tag}"])
        gr = OM.energy_gradient_fd(m)
        scale = np.max(np.abs(g[f"grad_{tag}"]))
        assert np.max(np.abs(gr - g[f"grad_{tag}"])) <= 1e-9 * scale
        assert np.max(np.abs(g[f"grad_{tag}"] - g[f"dense_grad_{tag}"])) <= 1e-8 * scale


def test_ih_fixture_reproduced_by_oracle():
    """The infinite-horizon model (steady-state gains from the warm-started
    Riccati recursions) after each of three lr = 0.9 VI steps, 1e-9."""
    from oracle import models as OM
    g = load("ih_m52_gaussian_N1000")
    sp = g["spec"]
    m = OM.InfiniteHorizonGP(oracle_kernel(sp["kernel"]), oracle_likelihood(sp["likelihood"]), g["x"], g["y"])
    for s in range(1, sp["steps"] + 1):
        m.inference(lr=sp["lr"], method="vi")
        assert rel_err(m.posterior_mean, g[f"mean_{s}"]) < 1e-9
        assert rel_err(m.posterior_variance, g[f"var_{s}"]) < 1e-9
        assert abs(m.energy("vi") - g[f"energy_{s}"]) <= 1e-9 * abs(g[f"energy_{s}"])


def test_meanfield_fixture_reproduced_and_equal_to_joint_model():
    """The mean-field model's block-diagonal filter and smoother reproduce the
    fixture (1e-9) and, with the diagonal VI sites, equal the joint model (1e-8)."""
    from oracle import models as OM
    g = load("meanfield_vi_hetero_N150")
    sp = g["spec"]
    m = OM.MarkovMeanFieldGP(oracle_kernel(sp["kernel"]), oracle_likelihood(sp["likelihood"]), g["x"], g["y"])
    for s in range(1, sp["steps"] + 1):
        m.inference(lr=sp["lr"], method="vi")
        assert rel_err(m.posterior_mean, g[f"mean_{s}"]) < 1e-9
        assert rel_err(m.posterior_variance, g[f"var_{s}"]) < 1e-9
        assert abs(m.energy("vi") - g[f"energy_{s}"]) <= 1e-9 * abs(g[f"energy_{s}"])
        assert rel_err(g[f"mean_{s}"], g[f"joint_mean_{s}"]) < 1e-8
        assert rel_err(g[f"var_{s}"], g[f"joint_var_{s}"]) < 1e-8
        assert abs(g[f"energy_{s}"] - g[f"joint_energy_{s}"]) <= 1e-9 * abs(g[f"joint_energy_{s}"])


def batch_series(g):
    """(kernel spec, likelihood spec, x, y, slice) of each series of the batch fixture."""
    o = g["offsets"]
    return [(["Matern32", float(g["variance"][i]), float(g["lengthscale"][i])], g["spec"]["likelihoods"][i],
             g["x"][o[i]:o[i + 1]], g["y"][o[i]:o[i + 1]], slice(int(o[i]), int(o[i + 1])))
            for i in range(len(o) - 1)]


def test_batch_fixture_reproduced_by_oracle_series_by_series():
    from oracle import models as OM
    g = load("batch_m32_mixed_S6")
    sp = g["spec"]
    for i, (ks, ls, x, y, sl) in enumerate(batch_series(g)):
        m = OM.MarkovGP(oracle_kernel(ks), oracle_likelihood(ls), x, y)
        for _ in range(sp["steps"]):
            m.inference(lr=sp["lr"])
        assert rel_err(m.posterior_mean.reshape(-1), g["mean"][sl]) < 1e-9, i
        assert rel_err(m.posterior_variance.reshape(-1), g["var"][sl]) < 1e-9, i
        assert abs(m.energy() - g["energy"][i]) <= 1e-9 * max(1.0, abs(g["energy"][i])), i
