"""Full-size parity: the bench workload (N = 1e6, Sum(Matern52, Matern32),
Bernoulli-logit, 20-point GH, parallel scan) in float32 against the float64 C++
restatement of the reference's sequential step (oracle/cpu_ref.cpp), after three
Newton steps; and a float64 GPU run of the same at N = 2e5.

Tolerances (normwise relative, max |diff| / max |oracle|): float32 posterior mean
1e-5 and variance 1e-4, energy 1e-6 relative; float64 1e-9.  The elementwise
relative error of the means (each entry against its own size, with a floor of
1e-3 of the largest) is reported beside the normwise one."""
import json
import os

import numpy as np
import pytest

from tests._cases import elem_rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

OUT = os.environ.get("BN_PARITY_OUT")


def _workload(N, seed=1):
    rng = np.random.default_rng(seed)
    x = np.sort(rng.uniform(0.0, 1e4 * N / 1e6, N))
    y = (rng.uniform(size=N) < 1.0 / (1.0 + np.exp(-2.0 * np.sin(x / 5.0)))).astype(np.float64)
    return x, y


def _rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("N,dtype,tol_m,tol_v,tol_e", [(1_000_000, "f32", 1e-5, 1e-4, 1e-6),
                                                     (200_000, "f64", 1e-9, 1e-9, 1e-10)])
def test_bench_workload_against_float64_port(N, dtype, tol_m, tol_v, tol_e):
    import bayesnewton_gb300 as bnx
    from oracle.cpu_ref import CpuRefModel
    x, y = _workload(N)
    dt = torch.float32 if dtype == "f32" else torch.float64
    kern = bnx.kernels.Sum([bnx.kernels.Matern52(1.0, 1.0), bnx.kernels.Matern32(1.0, 1.0)])
    gm = bnx.models.MarkovVariationalGP(kern, bnx.likelihoods.Bernoulli("logit"), x, y, dtype=dt)
    ref = CpuRefModel([("matern52", 1.0, 1.0), ("matern32", 1.0, 1.0)], 0, "logit", x, y)
    errs = []
    for step in range(3):
        gm.inference(lr=1.0)
        ref.step(newton=True, lr=1.0)
        pm = gm.posterior_mean[:, 0, 0].cpu().numpy()
        pv = gm.posterior_variance[:, 0, 0].cpu().numpy()
        e = gm.energy()
        errs.append({"step": step + 1, "mean": _rel(pm, ref.pm[:, 0]),
                     "mean_elementwise": elem_rel_err(pm, ref.pm[:, 0]), "var": _rel(pv, ref.pv[:, 0, 0]),
                     "energy": abs(e - ref.energy) / abs(ref.energy), "status": gm.status()})
    if OUT:
        with open(OUT, "a") as f:
            f.write(json.dumps({"N": N, "dtype": dtype, "errors": errs}) + "\n")
    for r in errs:
        assert r["mean"] < tol_m, errs
        assert r["var"] < tol_v, errs
        assert r["energy"] < tol_e, errs
