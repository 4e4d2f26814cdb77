"""bn_kalman_filter_noalloc: the allocation-free variant of the parallel Kalman
filter, for callers that cannot allocate device memory (a framework that owns all
allocations through its own arena, a loop that may not allocate after start-up).

Runs last (file name) so that a failure here leaves every other test already run.
It compares the variant with bn_kalman_filter, the entry point it mirrors, on two
calls in a row through the C ABI (the second on different data, so stale scratch
contents from the first call would show), within the float32 filter tolerance of
tests/test_gpu_ops.py (2e-5 relative), checks that each call writes its status
word (pre-filled with a sentinel; 0 on these healthy series), and that an
oversized call is rejected with BN_ERR_SCRATCH before anything runs."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 2e-5
ERR_SCRATCH = -4


def _entry(lib):
    f = lib.bn_kalman_filter_noalloc
    vp = ctypes.c_void_p
    from bayesnewton_gb300 import _lib
    f.argtypes = [ctypes.POINTER(_lib.PriorDesc), ctypes.c_int64, vp, ctypes.c_int32, vp, vp, vp, vp, vp, vp, vp, vp]
    f.restype = ctypes.c_int
    return f


def _inputs(N, seed, dev):
    rng = np.random.default_rng(seed)
    dt = np.concatenate([[0.0], rng.uniform(0.001, 0.05, N - 1)])
    y = rng.standard_normal(N)
    R = rng.uniform(0.05, 2.0, N)
    mask = (rng.uniform(size=N) < 0.05).astype(np.uint8)
    t = lambda a, d=torch.float32: torch.as_tensor(a, dtype=d, device=dev).contiguous()
    return t(dt), t(y).reshape(N, 1), t(R).reshape(N, 1, 1), t(mask, torch.uint8).reshape(N, 1)


def _rel(a, b):
    a, b = a.double().cpu().numpy(), b.double().cpu().numpy()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def test_noalloc_filter_matches_bn_kalman_filter_twice():
    import bayesnewton_gb300 as bnx
    from bayesnewton_gb300 import _lib
    lib = _lib.load()
    noalloc = _entry(lib)
    dev = torch.device("cuda", 0)
    kern = bnx.kernels.Sum([bnx.kernels.Matern52(1.0, 1.0), bnx.kernels.Matern32(1.0, 1.0)])
    desc = kern.desc()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call, (N, seed) in enumerate([(300_000, 1), (70_001, 2)]):
        dt, y, R, mask = _inputs(N, seed, dev)
        ell_ref, (m_ref, P_ref) = bnx.ops.kalman_filter(dt, kern, y, R, mask, parallel=True)
        means = torch.empty(N, 5, 1, dtype=torch.float32, device=dev)
        covs = torch.empty(N, 5, 5, dtype=torch.float32, device=dev)
        ell = torch.empty(1, dtype=torch.float64, device=dev)
        status = torch.full((1,), 0x7FFF, dtype=torch.int32, device=dev)
        rc = noalloc(ctypes.byref(desc), N, stream, 0, dt.data_ptr(), y.data_ptr(), R.data_ptr(), mask.data_ptr(),
                     means.data_ptr(), covs.data_ptr(), ell.data_ptr(), status.data_ptr())
        assert rc == 0, "call %d returned %d" % (call, rc)
        torch.cuda.synchronize()
        assert _rel(means, m_ref) < TOL, call
        assert _rel(covs, P_ref) < TOL, call
        assert abs(float(ell.item()) - ell_ref) <= TOL * max(1.0, abs(ell_ref)), (call, float(ell.item()), ell_ref)
        assert int(status.item()) == 0, (call, int(status.item()))


def test_noalloc_filter_rejects_oversized_call():
    import bayesnewton_gb300 as bnx
    from bayesnewton_gb300 import _lib
    lib = _lib.load()
    noalloc = _entry(lib)
    dev = torch.device("cuda", 0)
    desc = bnx.kernels.Sum([bnx.kernels.Matern52(1.0, 1.0), bnx.kernels.Matern32(1.0, 1.0)]).desc()
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = buf.data_ptr()
    # the size check runs before anything is launched or read
    rc = noalloc(ctypes.byref(desc), 10 ** 9, stream, 0, p, p, p, None, p, p, None, None)
    assert rc == ERR_SCRATCH
