"""GPU parity of the time-segmented step (one series cut into G segments, the
exchanges done in memory) against the unsplit model and the float64 oracle.
Tolerances as for the single-series models."""
import numpy as np
import pytest

from oracle import models as OM
from tests._cases import lik_pair, prior_pair, rel_err, series

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,prior,tol", [(torch.float64, "m52", 1e-9), (torch.float32, "sum52_32", 2e-4)])
@pytest.mark.parametrize("G", [2, 3, 5])
def test_segments_match_unsplit_model(dtype, prior, tol, G):
    import bayesnewton_gb300 as bnx
    from bayesnewton_gb300.segments import TimeSegment, run_segments
    ok, gk = prior_pair(prior)
    ol, gl = lik_pair("logit")
    x, y = series(3001, "logit", seed=11)
    segs = [TimeSegment(gk, gl, x, y, g, G, dtype=dtype, steps_per_thread=4) for g in range(G)]
    full = bnx.models.MarkovVariationalGP(gk, gl, x, y, dtype=dtype, steps_per_thread=4)
    om = OM.MarkovGP(ok, ol, x, y)
    run_segments(segs, False, 1.0)
    full.update_posterior()
    for _ in range(2):
        res = run_segments(segs, True, 1.0)
        full.inference(lr=1.0)
        om.inference(lr=1.0, method="vi")
    pm = torch.cat([s.model.posterior_mean.reshape(-1) for s in segs]).cpu()
    pv = torch.cat([s.model.posterior_variance.reshape(-1) for s in segs]).cpu()
    assert rel_err(pm, full.posterior_mean.reshape(-1).cpu()) < tol
    assert rel_err(pv, full.posterior_variance.reshape(-1).cpu()) < tol
    assert rel_err(pm, om.posterior_mean.reshape(-1)) < max(tol, 1e-8)
    e_full = full.energy()
    assert abs(res[0] - e_full) <= max(tol, 1e-9) * abs(e_full), (res[0], e_full)
    assert abs(res[0] - om.energy("vi", 1.0)) <= max(tol, 1e-8) * abs(e_full)
