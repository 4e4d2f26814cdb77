"""GPU parity of the ops-level filter and smoother (bayesnewton/ops.py:256-285,
:357-380) against the float64 oracle, through the C ABI.

Tolerances: float64 1e-9 relative (normwise: max |diff| / max |oracle|);
float32 2e-5 for the filter, 5e-5 for the smoother."""
import functools

import numpy as np
import pytest

from oracle import ops as OO
from tests._cases import prior_pair, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@functools.lru_cache(maxsize=None)
def _oracle(name, N, seed, masked):
    ok, _ = prior_pair(name)
    rng = np.random.default_rng(seed)
    P = ok.measurement_model().shape[0]
    dt = np.concatenate([[0.0], rng.uniform(0.01, 0.3, N - 1)])
    y = rng.standard_normal([N, P, 1])
    A = rng.uniform(-0.3, 0.3, [N, P, P])
    R = A @ np.swapaxes(A, 1, 2) + np.eye(P) * rng.uniform(0.05, 1.0, [N, 1, 1])
    mask = (rng.uniform(size=[N, P]) < 0.1) if masked else None
    ell, (fm, fP) = OO.kalman_filter(dt, ok, y, R, mask)
    dts = np.concatenate([dt[1:], [0.0]])
    sm, sP, G = OO.rauch_tung_striebel_smoother(dts, ok, fm, fP)
    smf, sPf, _ = OO.rauch_tung_striebel_smoother(dts, ok, fm, fP, return_full=True)
    _, (pm, pP) = OO.kalman_filter(dt, ok, y, R, mask, return_predict=True)
    return dict(dt=dt, y=y, R=R, mask=mask, ell=ell, fm=fm, fP=fP, dts=dts, sm=sm, sP=sP, G=G, smf=smf,
                sPf=sPf, pm=pm, pP=pP)


TOL = {torch.float64: (1e-9, 1e-9), torch.float32: (2e-5, 5e-5)}


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("parallel", [True, False])
@pytest.mark.parametrize("name", ["m12", "m32", "m52", "m72", "sum52_32", "sum32_12_32", "ind52_52", "ind32_32"])
@pytest.mark.parametrize("N", [1, 2, 3, 37, 1000, 4099])
def test_filter_smoother(dtype, parallel, name, N):
    import bayesnewton_gb300 as bnx
    if dtype == torch.float64 and name in ("m72", "m12", "sum32_12_32", "ind32_32"):
        pytest.skip("float64 is compiled for the layouts the configs use")
    ref = _oracle(name, N, 17 + N, True)
    _, kern = prior_pair(name)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.as_tensor(a, dtype=dtype, device=dev)
    mask = torch.as_tensor(ref["mask"], device=dev)
    ftol, stol = TOL[dtype]
    ell, (fm, fP) = bnx.ops.kalman_filter(t(ref["dt"]), kern, t(ref["y"]), t(ref["R"]), mask, parallel=parallel)
    assert abs(ell - ref["ell"]) <= ftol * max(1.0, abs(ref["ell"])) * 10
    assert rel_err(fm.cpu(), ref["fm"]) < ftol
    assert rel_err(fP.cpu(), ref["fP"]) < ftol
    _, (pm, pP) = bnx.ops.kalman_filter(t(ref["dt"]), kern, t(ref["y"]), t(ref["R"]), mask, parallel=parallel,
                                        return_predict=True)
    assert rel_err(pm.cpu(), ref["pm"]) < ftol
    assert rel_err(pP.cpu(), ref["pP"]) < ftol
    sm, sP, G = bnx.ops.rauch_tung_striebel_smoother(t(ref["dts"]), kern, t(ref["fm"]), t(ref["fP"]),
                                                     parallel=parallel)
    assert rel_err(sm.cpu(), ref["sm"]) < stol
    assert rel_err(sP.cpu(), ref["sP"]) < stol
    if N > 1:
        assert rel_err(G[:-1].cpu(), ref["G"][:-1]) < stol
    smf, sPf, _ = bnx.ops.rauch_tung_striebel_smoother(t(ref["dts"]), kern, t(ref["fm"]), t(ref["fP"]),
                                                       return_full=True, parallel=parallel)
    assert rel_err(smf.cpu(), ref["smf"]) < stol
    assert rel_err(sPf.cpu(), ref["sPf"]) < stol
