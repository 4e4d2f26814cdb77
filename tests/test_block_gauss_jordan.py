"""CPU model of the block Gauss-Jordan inverse that the spatio-temporal filter
combine runs on the GPU (`binv_reg_kernel` in bn_dense.cuh), in float64 numpy:
rows are never exchanged (pivot k takes the unused row with the largest |a_ik|,
compared by the float32 bit pattern of |a_ik|, smallest row on ties, or the
diagonal in order for symmetric positive definite input), each block of 4 pivots
is applied to its own 4 columns first (leaving the block transform's columns
T[:, P] there) and to every other column as x + (T[:, P] - I[:, P]) x_P, and the
stored result is unpermuted as inv(A)[pinv[i]][p_j] = S[i][j].  The kernel's own
float32 results are compared with numpy in tests/test_gpu_dense.py."""
import numpy as np
import pytest


def _key(v):
    return np.float32(abs(v)).view(np.uint32)


def block_gauss_jordan(A, width=4, spd=False):
    n = A.shape[0]
    S = np.array(A, dtype=np.float64)
    used = np.zeros(n, bool)
    perm, pinv = np.zeros(n, int), np.full(n, -1)
    for b0 in range(0, n, width):
        cols = list(range(b0, min(b0 + width, n)))
        old = S.copy()
        piv = []
        for s, k in enumerate(cols):
            if spd:
                p = k
            else:
                cand = [i for i in range(n) if not used[i]]
                p = max(cand, key=lambda i: (_key(S[i, k]), -i))
            prow = S[p, cols].copy()
            prow[s] = 1.0
            prow /= S[p, k]
            f = S[:, k].copy()
            S[:, k] = 0.0
            S[:, cols] -= np.outer(f, prow)
            S[p, cols] = prow
            used[p] = True
            perm[k], pinv[p] = p, k
            piv.append(p)
        G = S[:, cols].copy()
        for s, p in enumerate(piv):
            G[p, s] -= 1.0
        other = [j for j in range(n) if j not in cols]
        S[:, other] = old[:, other] + G @ old[piv][:, other]
    out = np.empty_like(S)
    out[np.ix_(pinv, perm)] = S
    return out, perm


@pytest.mark.parametrize("n", [1, 3, 4, 7, 13, 40])
def test_block_gauss_jordan_inverts(n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + 0.1 * np.eye(n)
    inv, _ = block_gauss_jordan(A)
    assert np.allclose(inv, np.linalg.inv(A), rtol=1e-9, atol=1e-9 * np.abs(np.linalg.inv(A)).max())


def test_pivot_rows_follow_partial_pivoting():
    """With the rows never exchanged, the chosen pivot rows are those the
    row-exchanging elimination would bring to each step (largest magnitude in the
    column among the rows not yet used)."""
    rng = np.random.default_rng(7)
    n = 12
    A = rng.standard_normal((n, n))
    _, perm = block_gauss_jordan(A)
    B = A.copy()
    rows = list(range(n))
    for k in range(n):
        p = max(range(k, n), key=lambda i: (abs(np.float32(B[i, k])), -rows[i]))
        B[[k, p]] = B[[p, k]]
        rows[k], rows[p] = rows[p], rows[k]
        assert perm[k] == rows[k]
        B[k + 1:] -= np.outer(B[k + 1:, k] / B[k, k], B[k])


def test_combine_matrix_form():
    """The combine's matrix I + C1 J2 (C1, J2 symmetric positive semi-definite, J2
    of low rank as at the scan's lowest level) at a width that leaves a ragged last
    block, and the diagonal-pivot mode on a symmetric positive definite matrix of
    condition 1e6."""
    rng = np.random.default_rng(3)
    n = 30
    G1, G2 = rng.standard_normal((n, n)), rng.standard_normal((n, 6))
    X = np.eye(n) + (G1 @ G1.T / n) @ (G2 @ G2.T)
    inv, _ = block_gauss_jordan(X)
    assert np.allclose(inv @ X, np.eye(n), atol=1e-9)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    P = (Q * np.geomspace(1e-3, 1e3, n)) @ Q.T
    inv, perm = block_gauss_jordan(P, spd=True)
    assert list(perm) == list(range(n))
    assert np.allclose(inv @ P, np.eye(n), atol=1e-6)


def test_nan_column_still_picks_an_unused_row():
    """A NaN entry is the largest key (its bit pattern is above infinity's), so the
    pivot choice stays a total order and always names an unused row."""
    A = np.eye(4)
    A[2, 0] = np.nan
    _, perm = block_gauss_jordan(A)
    assert perm[0] == 2
    assert sorted(perm) == [0, 1, 2, 3]
