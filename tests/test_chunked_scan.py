"""The library's chunked scan (tests/_chunked_scan.py, the work decomposition
of bayesnewton_gb300/csrc/bn_scan.cuh restated in float64 numpy) is exact: its
filtered and smoothed states and log marginal equal the oracle's sequential
filter and smoother (bayesnewton/ops.py:154-180, 288-311) for any chunk length,
and a chunk's element equals the composition of the reference's per-step
filter elements (ops.py:183-229) over the chunk.  Tolerances 1e-9 relative
(normwise), float64."""
import numpy as np
import pytest

from oracle import kernels as OK
from oracle import ops as OO
from tests import _chunked_scan as CS
from tests._cases import rel_err

PRIORS = {
    "m52": lambda: OK.Matern52(1.0, 1.0),
    "sum52_32": lambda: OK.Sum([OK.Matern52(1.0, 1.5), OK.Matern32(0.5, 4.0)]),
    "ind52_52": lambda: OK.Independent([OK.Matern52(1.0, 2.0), OK.Matern52(0.7, 5.0)]),
}


def _case(name, N, seed):
    kern = PRIORS[name]()
    P = kern.measurement_model().shape[0]
    rng = np.random.default_rng(seed)
    dt = np.concatenate([[0.0], rng.uniform(0.01, 0.3, N - 1)])
    if N > 6:
        dt[N // 3] = 0.0  # a repeated time point
    y = rng.standard_normal([N, P])
    B = rng.uniform(-0.3, 0.3, [N, P, P])
    R = B @ np.swapaxes(B, 1, 2) + np.eye(P) * rng.uniform(0.05, 1.0, [N, 1, 1])
    return kern, dt, y, R


@pytest.mark.parametrize("name", list(PRIORS))
@pytest.mark.parametrize("N,L", [(1, 4), (2, 1), (37, 4), (37, 32), (100, 8), (100, 100)])
def test_chunked_filter_and_smoother_equal_sequential(name, N, L):
    kern, dt, y, R = _case(name, N, 11 + N + L)
    ell_o, (fm_o, fP_o) = OO.kalman_filter(dt, kern, y[..., None], R)
    dts = np.concatenate([dt[1:], [0.0]])
    sm_o, sP_o, _ = OO.rauch_tung_striebel_smoother(dts, kern, fm_o, fP_o, return_full=True)
    ell, fm, fP, _ = CS.filter_chunked(dt, kern, y, R, L)
    assert abs(ell - ell_o) <= 1e-9 * max(1.0, abs(ell_o))
    assert rel_err(fm, fm_o[..., 0]) < 1e-9 and rel_err(fP, fP_o) < 1e-9
    sm, sP, at = CS.smoother_chunked(dt, kern, y, R, fm, fP, L)
    assert rel_err(sm, sm_o[..., 0]) < 1e-9 and rel_err(sP, sP_o) < 1e-9
    # the chunk-start states from the composed aggregates equal the reruns' states
    for s, (m, P) in at.items():
        assert rel_err(m, sm[s]) < 1e-9 and rel_err(P, sP[s]) < 1e-9


@pytest.mark.parametrize("name", list(PRIORS))
def test_chunk_element_equals_composed_reference_elements(name):
    """For a chunk [s, e) after the first step, the conditioned Kalman pass gives
    the same (A, b, C, J, eta) as composing the reference's per-step elements
    (ops.py:183-197) with the (I + C1 J2)^-1 combine."""
    kern, dt, y, R = _case(name, 40, 3)
    H, Pinf = kern.measurement_model(), kern.stationary_covariance()
    As = np.stack([kern.state_transition(float(d)) for d in dt])
    Qs = Pinf[None] - As @ Pinf[None] @ np.swapaxes(As, 1, 2)
    ref = OO.parallel_filtering_element(As, Qs, H, R, y[..., None])
    for s, e in [(5, 6), (5, 13), (17, 40)]:
        mine = CS.felem_identity(Pinf.shape[0])
        for k in range(s, e):
            mine = CS.felem_step(mine, As[k], Pinf, H, y[k], R[k])
        tot = [x[s] for x in ref]
        for k in range(s + 1, e):
            tot = OO.parallel_filtering_operator_stable(tot, [x[k] for x in ref])
        for a, b in zip(mine, tot):
            b = np.asarray(b).reshape(np.shape(a))
            assert np.max(np.abs(a - b)) <= 1e-10 * max(1.0, np.max(np.abs(b)))


@pytest.mark.parametrize("fixture", ["vi_m52_gaussian_N400", "vi_sum52_32_logit_N500"])
@pytest.mark.parametrize("L", [4, 32])
def test_chunked_scan_at_dense_input_spacing(fixture, L):
    """At the golden fixtures' input spacing (0.01 at lengthscale 1), where the
    reference's own parallel combine fails, the chunked decomposition still
    equals the sequential filter and smoother (1e-12)."""
    from tests.golden.spec import oracle_kernel
    from tests.test_golden import load
    g = load(fixture)
    kern = oracle_kernel(g["spec"]["kernel"])
    x = g["x"]
    N = x.shape[0]
    dt = np.concatenate([[0.0], np.diff(x)])
    rng = np.random.default_rng(0)
    y = rng.standard_normal([N, 1])
    R = rng.uniform(0.05, 10.0, [N, 1, 1])
    ell_o, (fm_o, fP_o) = OO.kalman_filter(dt, kern, y[..., None], R)
    dts = np.concatenate([dt[1:], [0.0]])
    sm_o, sP_o, _ = OO.rauch_tung_striebel_smoother(dts, kern, fm_o, fP_o, return_full=True)
    ell, fm, fP, _ = CS.filter_chunked(dt, kern, y, R, L)
    sm, sP, _ = CS.smoother_chunked(dt, kern, y, R, fm, fP, L)
    assert abs(ell - ell_o) <= 1e-12 * abs(ell_o)
    assert rel_err(fm, fm_o[..., 0]) < 1e-12 and rel_err(fP, fP_o) < 1e-12
    assert rel_err(sm, sm_o[..., 0]) < 1e-12 and rel_err(sP, sP_o) < 1e-12


def test_float32_error_at_the_heteroscedastic_spacing_comes_from_q():
    """Float32 emulation of the filter and smoother (numpy float32, no fused
    multiply-adds) on the two-latent heteroscedastic workload's prior
    (Independent(Matern52(1, 10), Matern52(0.25, 20))) at its input spacing
    (0.005, dt / lengthscale ~ 5e-4) with heteroscedastic-like site variances:
    the posterior means are ~1e-4 off float64 with the prediction in its Pinf
    form A (P - Pinf) A^T + Pinf (rounding of order eps |Pinf| against a filtered
    P far below Pinf), and below 2e-5 with A P A^T + Q, A and Q formed in
    float64 and rounded.  At the long-series spacing (Sum(Matern52, Matern32),
    lengthscale 1, spacing 0.01) the Q form does not matter (both below 1e-5)."""
    cases = [(OK.Independent([OK.Matern52(1.0, 10.0), OK.Matern52(0.25, 20.0)]), 0.005, (0.5, 5.0), 2),
             (OK.Sum([OK.Matern52(1.0, 1.0), OK.Matern32(1.0, 1.0)]), 0.01, (4.0, 10.0), 1)]
    errs = []
    for kern, spacing, (rlo, rhi), P in cases:
        rng = np.random.default_rng(0)
        N = 5000
        x = np.sort(rng.uniform(0.0, N * spacing, N))
        dt = np.concatenate([[0.0], np.diff(x)])
        y = rng.standard_normal([N, P])
        R = np.zeros([N, P, P])
        for p in range(P):
            R[:, p, p] = rng.uniform(rlo, rhi, N)
        ref = CS.sequential_posterior_mean(dt, kern, y, R)
        e32 = rel_err(CS.sequential_posterior_mean(dt, kern, y, R, np.float32), ref)
        e32q = rel_err(CS.sequential_posterior_mean(dt, kern, y, R, np.float32, q_float64=True), ref)
        e32l = rel_err(CS.sequential_posterior_mean(dt, kern, y, R, np.float32, q_float64="library"), ref)
        errs.append((e32, e32q, e32l))
    (h32, h32q, h32l), (l32, l32q, l32l) = errs
    assert h32 > 5e-5 and h32q < 2e-5 and h32 > 5 * h32q, errs
    assert l32 < 1e-5 and l32q < 1e-5, errs
    # the library's float32 A and Q (cancellation-free Q) do as well as float64 ones
    assert h32l < 2e-5 and h32 > 5 * h32l and l32l < 1e-5, errs


def test_float32_chunked_scan_with_float64_q():
    """The same comparison through the chunked decomposition the GPU runs
    (chunk length 32) at the heteroscedastic workload's spacing: the float32
    posterior means improve by more than 5x with A P A^T + Q (A, Q in float64),
    and as much with the float32 A and Q the library's kernels form
    (bn_matern_process_noise)."""
    kern = OK.Independent([OK.Matern52(1.0, 10.0), OK.Matern52(0.25, 20.0)])
    rng = np.random.default_rng(0)
    N = 4000
    x = np.sort(rng.uniform(0.0, N * 0.005, N))
    dt = np.concatenate([[0.0], np.diff(x)])
    y = rng.standard_normal([N, 2])
    R = np.zeros([N, 2, 2])
    R[:, 0, 0], R[:, 1, 1] = rng.uniform(0.5, 5.0, N), rng.uniform(0.5, 5.0, N)
    H = kern.measurement_model()
    _, fm, fP, _ = CS.filter_chunked(dt, kern, y, R, 32)
    sm, _, _ = CS.smoother_chunked(dt, kern, y, R, fm, fP, 32)
    ref = sm @ H.T
    err = {}
    for q in (False, True, "library"):
        _, fm, fP, _ = CS.filter_chunked(dt, kern, y, R, 32, np.float32, q_float64=q)
        sm, _, _ = CS.smoother_chunked(dt, kern, y, R, fm, fP, 32, np.float32, q_float64=q)
        err[q] = rel_err(sm.astype(np.float64) @ H.T, ref)
    assert err[False] > 5 * err[True] and err[True] < 2e-5, err
    assert err[False] > 5 * err["library"] and err["library"] < 2e-5, err
