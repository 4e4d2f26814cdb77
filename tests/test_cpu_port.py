"""The float64 C++ restatement (oracle/cpu_ref.cpp: the timed CPU baseline and
the large-N oracle of the GPU tests) against the numpy oracle's committed golden
fixtures and the plain workload at full size: posterior means, (co)variances and
energies after the same VI steps, 1e-9 relative (normwise)."""
import numpy as np
import pytest

from tests._cases import rel_err
from tests.test_golden import batch_series, load

LIK = {"Gaussian": "gaussian", "Poisson": "poisson", "HeteroscedasticNoise": "hetero_exp"}


def _port(kernel_spec, lik_spec, x, y):
    from oracle.cpu_ref import CpuRefModel
    if kernel_spec[0] in ("Sum", "Independent"):
        comps, combine = kernel_spec[1:], 1 if kernel_spec[0] == "Independent" else 0
    else:
        comps, combine = [kernel_spec], 0
    comps = [(c[0].lower(), float(c[1]), float(c[2])) for c in comps]
    name = lik_spec[1] if lik_spec[0] == "Bernoulli" else LIK[lik_spec[0]]
    if lik_spec[0] == "HeteroscedasticNoise":
        name = "hetero_" + lik_spec[1]
    var = float(lik_spec[1]) if lik_spec[0] == "Gaussian" else 1.0
    return CpuRefModel(comps, combine, name, x, y, lik_variance=var, threads=1)


@pytest.mark.parametrize("name", ["vi_m52_gaussian_N400", "vi_sum52_32_logit_N500", "vi_m32_poisson_N300",
                                  "vi_hetero_exp_N150"])
def test_port_matches_golden_fixture(name):
    g = load(name)
    sp = g["spec"]
    m = _port(sp["kernel"], sp["likelihood"], g["x"], g["y"])
    for s in range(1, sp["steps"] + 1):
        m.step(newton=True, lr=sp["lr"])
        assert rel_err(m.pm, g[f"mean_{s}"].reshape(m.pm.shape)) < 1e-9, s
        assert rel_err(m.pv, g[f"var_{s}"].reshape(m.pv.shape)) < 1e-9, s
        assert abs(m.energy - g[f"energy_{s}"]) <= 1e-9 * abs(g[f"energy_{s}"]), (s, m.energy, g[f"energy_{s}"])


def test_port_matches_golden_batch_series():
    g = load("batch_m32_mixed_S6")
    sp = g["spec"]
    for i, (ks, ls, x, y, sl) in enumerate(batch_series(g)):
        m = _port(ks, ls, x, y)
        for _ in range(sp["steps"]):
            m.step(newton=True, lr=sp["lr"])
        assert rel_err(m.pm.reshape(-1), g["mean"][sl]) < 1e-9, i
        assert rel_err(m.pv.reshape(-1), g["var"][sl]) < 1e-9, i
        assert abs(m.energy - g["energy"][i]) <= 1e-9 * max(1.0, abs(g["energy"][i])), i


def test_port_matches_oracle_on_the_plain_workload():
    from tests._plain_config import plain_data, plain_oracle
    x, y = plain_data()
    om, ov, oe = plain_oracle()
    m = _port(["Matern52", 1.0, 1.0], ["Gaussian", 0.1], x, y)
    m.step(newton=True, lr=1.0)
    assert rel_err(m.pm, om.reshape(m.pm.shape)) < 1e-9
    assert rel_err(m.pv, ov.reshape(m.pv.shape)) < 1e-9
    assert abs(m.energy - oe) <= 1e-10 * abs(oe)
