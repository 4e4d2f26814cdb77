"""Full-size parity of the spatio-temporal VI step: the workload of bench.py
--workload st (Nt = 2,000 unit-spaced time points, M = 100 inducing inputs on a
10 x 10 grid, state dimension 200, 500 observations per time point, Matern32 in
time (lengthscale 20) x Matern32 in space (lengthscale 0.3), Poisson counts with
f drawn from the prior), float32 on the device, against the float64 numpy
restatement of the reference's spatio-temporal path (oracle/spatiotemporal.py;
kernels.py:385-586, basemodels.py:676-764) on the same inputs, after the
workload's VI step at lr = 1 from the initial sites.

Tolerances: 5e-4 normwise relative on the data-space marginal means and
variances and on the latent posterior (the spatio-temporal tolerance of
tests/test_gpu_spatiotemporal.py); 1e-4 relative on the energy, a sum of 1e6
Poisson terms of magnitude ~300 formed in float32 (measured: means 3e-6 data
space, 1e-5 latent; variances 1e-5 / 3e-5; energy 2.8e-5).

A second step is not compared at this size: from the first step's sites the
float64 iteration drives the largest counts' site precisions exp(m + v/2) beyond
1e6 times the prior precision (at lr = 1 and at lr = 0.5 alike), where the
float32 filter update loses the site variance's digits; the float32 path clamps
those sites and reports it (BN_STATUS_SITE_CLAMPED), which the test checks,
instead of following the float64 iteration (measured after such a step: 2e-2 on
the data-space means).  The measured errors are printed (and appended to
BN_PARITY_OUT when set) beside the assertions."""
import json
import os

import numpy as np
import pytest

from tests._cases import elem_rel_err, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL, ETOL = 5e-4, 1e-4
OUT = os.environ.get("BN_PARITY_OUT")


def test_spatiotemporal_workload_against_float64_oracle():
    import bayesnewton_gb300 as bnx
    from bench import st_workload
    from oracle import kernels as OK
    from oracle import likelihoods as OL
    from oracle.spatiotemporal import SpatioTemporalKernel as OSTK
    from oracle.spatiotemporal import STMarkovGP
    z, X, R, Y, lt, ls = st_workload()
    gk = bnx.kernels.SpatioTemporalMatern32(1.0, lt, ls, z=z)
    gm = bnx.models.MarkovVariationalGP(gk, bnx.likelihoods.Poisson(), X, Y, R=R)
    om = STMarkovGP(OSTK(OK.Matern32(1.0, lt), OK.Matern32(1.0, ls), z), OL.Poisson(), X, R, Y)
    errs = []
    gm.inference(lr=1.0)
    om.inference(lr=1.0)
    mf, vf = om.conditional_posterior_to_data()
    e_g, e_o = gm.energy(), om.energy()
    r = {"step": 1, "lr": 1.0,
         "data_mean": rel_err(gm.data_mean.cpu(), mf),
         "data_mean_elementwise": elem_rel_err(gm.data_mean.cpu(), mf),
         "data_var": rel_err(gm.data_variance.cpu(), vf),
         "latent_mean": rel_err(gm.posterior_mean.cpu(), om.posterior_mean),
         "latent_var": rel_err(gm.posterior_variance.cpu(), om.posterior_variance),
         "energy": abs(e_g - e_o) / abs(e_o), "status": gm.status()}
    errs.append(r)
    # the second step: the float32 range guard reports the clamped sites
    gm.inference(lr=1.0)
    st2 = gm.status()
    errs.append({"step": 2, "lr": 1.0, "status": st2})
    print(json.dumps(errs))
    if OUT:
        with open(OUT, "a") as f:
            f.write(json.dumps({"workload": "spatio-temporal Nt=2000 M=100 Nr=500", "errors": errs}) + "\n")
    for k in ("data_mean", "data_var", "latent_mean", "latent_var"):
        assert r[k] < TOL, errs
    assert r["energy"] < ETOL, errs
    assert r["status"] == 0, errs
    assert st2 & 8, errs  # BN_STATUS_SITE_CLAMPED
