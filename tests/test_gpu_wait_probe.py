"""Failure detection without a GPU fault: a device wait that nothing satisfies
gives up after its poll limit and reports it, the kernel returns, and the
context keeps running the library's kernels.

bn_bounded_wait_probe runs the bounded mbarrier poll loop of the tensor-core
kernels on a phase that no one completes (it must give up) and on a phase it
completes itself (it must succeed).  Afterwards an ops-level filter on the same
context still matches the float64 oracle (float32 tolerance 2e-5, as in
tests/test_gpu_ops.py)."""
import ctypes

import numpy as np
import pytest

from oracle import ops as OO
from tests._cases import prior_pair, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_wait_gives_up_reports_and_context_stays_usable(lib):
    import bayesnewton_gb300 as bnx
    dev = torch.device("cuda", 0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for polls in (256, 4096):
        status = torch.zeros(2, dtype=torch.int32, device=dev)
        assert lib.bn_bounded_wait_probe(stream, polls, ctypes.c_void_p(status.data_ptr())) == 0
        torch.cuda.synchronize()
        assert status.tolist() == [1, 1], (polls, status.tolist())
    ok, kern = prior_pair("m52")
    rng = np.random.default_rng(5)
    N = 257
    dt = np.concatenate([[0.0], rng.uniform(0.01, 0.3, N - 1)])
    y = rng.standard_normal([N, 1, 1])
    R = rng.uniform(0.05, 1.0, [N, 1, 1])
    ell_o, (fm_o, fP_o) = OO.kalman_filter(dt, ok, y, R)
    t = lambda a: torch.as_tensor(a, dtype=torch.float32, device=dev)  # noqa: E731
    mask = torch.zeros(N, 1, dtype=torch.uint8, device=dev)
    ell, (fm, fP) = bnx.ops.kalman_filter(t(dt), kern, t(y), t(R), mask, parallel=True)
    assert rel_err(fm.cpu(), fm_o) < 2e-5
    assert rel_err(fP.cpu(), fP_o) < 2e-5
    assert abs(ell - ell_o) <= 2e-4 * max(1.0, abs(ell_o))
