"""The batched products behind the spatio-temporal path on both engines -- the
tcgen05 tensor-core kernel (TMA-fed, 3xTF32: TF32 heads and float32 remainders,
float32 accumulation in tensor memory) and the CUDA-core tiles -- against float64,
for every transpose combination, ragged tile edges (rows, columns and K slices
that end inside a tile, a row count that spills into a third row tile, a
column count that spills into a third column tile) and the shapes the tensor-core
kernel turns down."""
import ctypes

import numpy as np
import pytest

from tests._cases import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _tma_ok(ta, tb, M, N, K):
    """the tensor-core kernel's operand boxes need whole 16-byte units along each
    operand's contiguous extent"""
    return (M if ta else K) % 4 == 0 and (K if tb else N) % 4 == 0


@pytest.mark.parametrize("tc", [1, 0])
@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("M,N,K", [(200, 200, 200), (100, 200, 100), (132, 76, 44), (260, 228, 36), (130, 70, 44),
                                   (130, 70, 45)])
def test_batched_gemm_matches_float64(tc, ta, tb, M, N, K):
    from bayesnewton_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(M + N + K)
    batch = 3
    A = rng.standard_normal((batch, K, M) if ta else (batch, M, K)).astype(np.float32)
    B = rng.standard_normal((batch, N, K) if tb else (batch, K, N)).astype(np.float32)
    C0 = rng.standard_normal((batch, M, N)).astype(np.float32)
    ref = 0.7 * np.einsum("bij,bjk->bik", (A.transpose(0, 2, 1) if ta else A).astype(np.float64),
                          (B.transpose(0, 2, 1) if tb else B).astype(np.float64)) + 0.3 * C0.astype(np.float64)
    dA, dB, dC0 = (torch.as_tensor(x, device="cuda") for x in (A, B, C0))
    dC = torch.empty(batch, M, N, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    rc = lib.bn_dense_gemm(ctypes.c_void_p(s), tc, batch, ta, tb, M, N, K, 0.7, ctypes.c_void_p(dA.data_ptr()),
                           ctypes.c_void_p(dB.data_ptr()), 0.3, ctypes.c_void_p(dC0.data_ptr()),
                           ctypes.c_void_p(dC.data_ptr()))
    if tc and not _tma_ok(ta, tb, M, N, K):
        assert rc == -1  # BN_ERR_ARG: the bgemm dispatcher takes the CUDA-core tiles for these
        return
    assert rc == 0
    torch.cuda.synchronize()
    # float32-level accuracy: 3xTF32 and the float32 FMA tiles alike
    assert rel_err(dC.cpu().numpy(), ref) < 2e-6 * np.sqrt(K)


def test_engines_agree_at_spatiotemporal_size():
    """1024 products of 200 x 200 x 200 (the shape of one spatio-temporal scan
    level): both engines against each other over the whole batch and against
    float64 on a sample of it."""
    from bayesnewton_gb300 import _lib
    lib = _lib.load()
    batch, n = 1024, 200
    g = torch.Generator(device="cuda").manual_seed(0)
    dA = torch.randn(batch, n, n, device="cuda", generator=g)
    dB = torch.randn(batch, n, n, device="cuda", generator=g)
    s = torch.cuda.current_stream().cuda_stream
    out = []
    for tc in (1, 0):
        dC = torch.empty(batch, n, n, device="cuda")
        for _ in range(2):
            assert lib.bn_dense_gemm(ctypes.c_void_p(s), tc, batch, 0, 0, n, n, n, 1.0,
                                     ctypes.c_void_p(dA.data_ptr()), ctypes.c_void_p(dB.data_ptr()), 0.0, None,
                                     ctypes.c_void_p(dC.data_ptr())) == 0
        out.append(dC)
    torch.cuda.synchronize()
    assert float((out[0] - out[1]).abs().max()) < 4e-6 * np.sqrt(n) * float(out[1].abs().max())
    idx = [0, 511, 1023]
    ref = torch.bmm(dA[idx].double(), dB[idx].double())
    for o in out:
        assert rel_err(o[idx].cpu().numpy(), ref.cpu().numpy()) < 2e-6 * np.sqrt(n)


@pytest.mark.parametrize("engine", [1, 0])
@pytest.mark.parametrize("n", [200, 131, 64, 7, 1])
def test_batched_inverse_matches_float64(engine, n):
    """Both Gauss-Jordan kernels against float64 on matrices of the spatio-temporal
    combine's form, I + C1 J2 (C1, J2 symmetric positive semi-definite), plus one
    matrix that needs row pivoting (zero leading diagonal) and one singular matrix
    (status bit, no fault); log|det| from the pivots."""
    from bayesnewton_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(n)
    batch = 5
    mats = []
    for _ in range(batch - 2):
        G1, G2 = rng.standard_normal((n, n)), rng.standard_normal((n, n))
        C1, J2 = G1 @ G1.T / n, G2 @ G2.T / n
        mats.append(np.eye(n) + C1 @ J2)
    P = rng.standard_normal((n, n)) + n * np.eye(n)
    P[[0, n - 1]] = P[[n - 1, 0]]  # the largest entries off the diagonal in the first and last rows
    mats.append(P)
    mats.append(np.zeros((n, n)))
    A = np.stack(mats).astype(np.float32)
    dA = torch.as_tensor(A, device="cuda")
    ld = torch.zeros(batch, dtype=torch.float64, device="cuda")
    stt = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    rc = lib.bn_dense_inverse(ctypes.c_void_p(s), engine, batch, n, ctypes.c_void_p(dA.data_ptr()),
                              ctypes.c_void_p(ld.data_ptr()), ctypes.c_void_p(stt.data_ptr()))
    assert rc == 0
    torch.cuda.synchronize()
    assert int(stt.item()) == 1  # the zero matrix
    out = dA.cpu().numpy().astype(np.float64)
    for b in range(batch - 1):
        ref = np.linalg.inv(A[b].astype(np.float64))
        cond = np.linalg.cond(A[b].astype(np.float64))
        assert rel_err(out[b], ref) < 2e-6 * max(1.0, cond) * np.sqrt(n), b
        sign, lref = np.linalg.slogdet(A[b].astype(np.float64))
        assert abs(float(ld[b].item()) - lref) < 1e-4 * max(1.0, abs(lref)) + 1e-4, b


@pytest.mark.parametrize("n", [200, 96, 5])
def test_spd_inverse_without_pivot_search(n):
    """The register-resident inverse with the diagonal pivots in order (engine 2, the
    smoother gains' Pp^-1) against float64 on symmetric positive definite matrices
    of a wide spread of eigenvalues, and a singular one flagged in the status."""
    from bayesnewton_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(100 + n)
    mats = []
    for scale in (1e-3, 1.0, 30.0):
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        ev = np.geomspace(1.0, 1e3, n) * scale
        mats.append((Q * ev) @ Q.T)
    mats.append(np.zeros((n, n)))
    A = np.stack(mats).astype(np.float32)
    dA = torch.as_tensor(A, device="cuda")
    ld = torch.zeros(len(mats), dtype=torch.float64, device="cuda")
    stt = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert lib.bn_dense_inverse(ctypes.c_void_p(s), 2, len(mats), n, ctypes.c_void_p(dA.data_ptr()),
                                ctypes.c_void_p(ld.data_ptr()), ctypes.c_void_p(stt.data_ptr())) == 0
    torch.cuda.synchronize()
    assert int(stt.item()) == 1
    out = dA.cpu().numpy().astype(np.float64)
    for b in range(len(mats) - 1):
        A64 = A[b].astype(np.float64)
        ref = np.linalg.inv(A64)
        assert rel_err(out[b], ref) < 2e-6 * np.linalg.cond(A64) * np.sqrt(n), b
        assert abs(float(ld[b].item()) - np.linalg.slogdet(A64)[1]) < 1e-4 * n, b
