"""float64 numpy model of the library's chunked scan (the work decomposition of
bayesnewton_gb300/csrc/bn_scan.cuh), used by tests/test_chunked_scan.py to show
on the CPU that the reorganisation is exact: it reproduces the oracle's
sequential filter and smoother (bayesnewton/ops.py:154-180, 288-311).

Filter: each chunk [s, e) of L steps forms its element (A, b, C, J, eta) by a
Kalman pass conditioned on a known x_{s-1} (predict M <- A M, b <- A b,
C <- A (C - Pinf) A^T + Pinf, then a Kalman update of (M x + b, C) that also
accumulates the information J, eta about x_{s-1}); chunk elements are combined
with W = (I + C1 J2)^-1 (no inverse of C1); each chunk then reruns the ordinary
filter from the exact filtered state entering it.

Smoother: each chunk's aggregate (E, g, L) of its RTS elements comes from a
fixed-point smoother of the chunk's first state carried through the chunk
(X = Cov(x_s, x_k | y_..k), mu, Sig), closed at the chunk end with the joint
Gaussian of (x_s, x_e); aggregates compose backwards, and each chunk reruns
sm_k = E_k sm_{k+1} + g_k, sP_k = E_k sP_{k+1} E_k^T + L_k from the exact
smoothed state after it."""
import numpy as np


def _library_aq(dt, kernel):
    """Per-step float32 A and Q of a prior made of Matern blocks, as the library's
    float32 kernels form them (bn_matern_process_noise: Q without the cancellation
    of Pinf - A Pinf A^T)."""
    import ctypes
    from bayesnewton_gb300 import _lib
    lib = _lib.load()
    f = lib.bn_matern_process_noise
    f.argtypes = [ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                  ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    f.restype = ctypes.c_int
    comps = getattr(kernel, "kernels", [kernel])
    D = sum(k.state_dim for k in comps)
    A = np.zeros((len(dt), D, D), np.float32)
    Q = np.zeros((len(dt), D, D), np.float32)
    o = 0
    for k in comps:
        S = k.state_dim
        a = (ctypes.c_float * (S * S))()
        q = (ctypes.c_float * (S * S))()
        for n, d in enumerate(dt):
            assert f(S, k.variance, k.lengthscale, float(d), a, q) == 0
            A[n, o:o + S, o:o + S] = np.array(a[:], np.float32).reshape(S, S)
            Q[n, o:o + S, o:o + S] = np.array(q[:], np.float32).reshape(S, S)
        o += S
    return A, Q


def _transitions(dt, kernel, dtype=np.float64, q_float64=False):
    """Per-step A (A[0] = I: the first step starts from the stationary prior) and,
    with q_float64, Q = Pinf - A Pinf A^T formed in float64; both rounded to dtype.
    q_float64 = "library": A and Q as the library's float32 kernels form them."""
    if q_float64 == "library":
        d = np.array(dt, np.float64)
        d[0] = 0.0  # A_0 = I, Q_0 = 0
        A, Q = _library_aq(d, kernel)
        return A.astype(dtype), Q.astype(dtype)
    A64 = np.stack([kernel.state_transition(float(d)) for d in dt])
    A64[0] = np.eye(A64.shape[1])
    if not q_float64:
        return A64.astype(dtype), None
    Pinf = kernel.stationary_covariance()
    Q64 = Pinf[None] - A64 @ Pinf[None] @ np.swapaxes(A64, 1, 2)
    return A64.astype(dtype), Q64.astype(dtype)


def _pred(A, P, Pinf, Q):
    """Predicted covariance: the Pinf form A (P - Pinf) A^T + Pinf of the float32
    kernels, or A P A^T + Q when Q is given."""
    return A @ P @ A.T + Q if Q is not None else A @ (P - Pinf) @ A.T + Pinf


def felem_identity(D, dtype=np.float64):
    return [np.eye(D, dtype=dtype), np.zeros(D, dtype), np.zeros((D, D), dtype), np.zeros((D, D), dtype),
            np.zeros(D, dtype)]


def felem_step(e, A, Pinf, H, y, R, Q=None):
    """One step of the chunk element: a Kalman step conditioned on x_{s-1}."""
    M, b, C, J, eta = e
    M = A @ M
    b = A @ b
    Cp = _pred(A, C, Pinf, Q)
    HM, HC = H @ M, H @ Cp
    S = HC @ H.T + R
    Si = np.linalg.inv(S)
    r = y - H @ b
    eta = eta + HM.T @ Si @ r
    J = J + HM.T @ Si @ HM
    K = HC.T @ Si
    return [M - K @ HM, b + K @ r, Cp - K @ HC, J, eta]


def fcombine(e1, e2):
    """e1 (earlier) then e2 (later), with W = (I + C1 J2)^-1."""
    A1, b1, C1, J1, eta1 = e1
    A2, b2, C2, J2, eta2 = e2
    W = np.linalg.inv(np.eye(A1.shape[0], dtype=A1.dtype) + C1 @ J2)
    A2W = A2 @ W
    WA1 = W @ A1
    return [A2W @ A1, A2W @ (b1 + C1 @ eta2) + b2, A2W @ C1 @ A2.T + C2,
            WA1.T @ J2 @ A1 + J1, WA1.T @ (eta2 - J2 @ b1) + eta1]


def state_fcombine(m, P, e):
    """A filtered state followed by an element."""
    A, b, C, J, eta = e
    W = np.linalg.inv(np.eye(A.shape[0], dtype=A.dtype) + P @ J)
    AW = A @ W
    return AW @ (m + P @ eta) + b, AW @ P @ A.T + C


def _kf_step(m, P, A, Pinf, H, y, R, Q=None):
    mp = A @ m
    Pp = _pred(A, P, Pinf, Q)
    S = H @ Pp @ H.T + R
    K = np.linalg.solve(S, H @ Pp).T
    r = y - H @ mp
    ell = -0.5 * float(r @ np.linalg.solve(S, r) + np.linalg.slogdet(2 * np.pi * S)[1])
    return mp + K @ r, Pp - K @ S @ K.T, mp, Pp, ell


def filter_chunked(dt, kernel, y, R, L, dtype=np.float64, q_float64=False):
    """Filtered means [N, D], covariances [N, D, D] and the log marginal, by
    chunk elements -> exclusive prefix over chunks -> chunk reruns.  The first
    step starts from the stationary prior (A_0 = I, Q_0 = 0 from (0, Pinf)).
    dtype: the arithmetic type of every array (float32 emulates the bulk
    precision of the float32 path, without its fused multiply-adds); q_float64:
    predictions A P A^T + Q with A and Q formed in float64."""
    N = dt.shape[0]
    H = kernel.measurement_model().astype(dtype)
    Pinf = kernel.stationary_covariance().astype(dtype)
    D = Pinf.shape[0]
    A, Q = _transitions(dt, kernel, dtype, q_float64)
    Qk = (lambda k: Q[k]) if Q is not None else (lambda k: None)  # noqa: E731
    y = y.reshape(N, -1).astype(dtype)
    R = R.reshape(N, y.shape[1], y.shape[1]).astype(dtype)
    starts = list(range(0, N, L))
    elems = []
    for s in starts:
        e = felem_identity(D, dtype)
        for k in range(s, min(s + L, N)):
            e = felem_step(e, A[k], Pinf, H, y[k], R[k], Qk(k))
        elems.append(e)
    # exclusive prefix: the filtered state entering each chunk
    m, P = np.zeros(D, dtype), Pinf.copy()
    entering = []
    for e in elems:
        entering.append((m, P))
        m, P = state_fcombine(m, P, e)
    fm, fP, ell = np.zeros((N, D), dtype), np.zeros((N, D, D), dtype), 0.0
    for s, (m, P) in zip(starts, entering):
        for k in range(s, min(s + L, N)):
            m, P, _, _, lk = _kf_step(m, P, A[k], Pinf, H, y[k], R[k], Qk(k))
            fm[k], fP[k] = m, P
            ell += lk
    return ell, fm, fP, elems


def chunk_smoother_aggregate(fm, fP, A, Pinf, H, y, R, s, e, Q=None):
    """(E, g, L) of x_s given x_e over the chunk [s, e), from the fixed-point
    smoother of x_s carried through the chunk's filter steps.  A[k] maps k-1 to
    k (the filter's transitions); (fm, fP)[s] is the filtered state at s."""
    mu, Sig, X = fm[s].copy(), fP[s].copy(), fP[s].copy()
    for k in range(s + 1, e):
        Xm = X @ A[k].T
        Pp = _pred(A[k], fP[k - 1], Pinf, None if Q is None else Q[k])
        mp = A[k] @ fm[k - 1]
        S = H @ Pp @ H.T + R[k]
        Si = np.linalg.inv(S)
        c = Xm @ H.T
        r = y[k] - H @ mp
        mu = mu + c @ Si @ r
        Sig = Sig - c @ Si @ c.T
        X = Xm - c @ Si @ H @ Pp
    Ce = X @ A[e].T
    Ppe = _pred(A[e], fP[e - 1], Pinf, None if Q is None else Q[e])
    mpe = A[e] @ fm[e - 1]
    E = Ce @ np.linalg.inv(Ppe)
    return E, mu - E @ mpe, Sig - E @ Ce.T


def smoother_chunked(dt, kernel, y, R, fm, fP, L, dtype=np.float64, q_float64=False):
    """Smoothed means / covariances [N, D] / [N, D, D] from the filtered states:
    chunk aggregates composed backwards give the smoothed state at every chunk
    start (the last chunk's aggregate closes at the last time point, whose
    smoothed state is its filtered state); each chunk then reruns its per-step
    RTS elements from the smoothed state after it.  dt is the filter's (A[k]
    maps k-1 to k).  Returns (sm, sP, chunk-start states from the aggregates)."""
    N = dt.shape[0]
    H = kernel.measurement_model().astype(dtype)
    Pinf = kernel.stationary_covariance().astype(dtype)
    D = Pinf.shape[0]
    A, Q = _transitions(dt, kernel, dtype, q_float64)
    y = y.reshape(N, -1).astype(dtype)
    R = R.reshape(N, y.shape[1], y.shape[1]).astype(dtype)
    fm, fP = fm.astype(dtype), fP.astype(dtype)
    starts = list(range(0, N, L))
    ends = starts[1:] + [N - 1]
    state_at = {N - 1: (fm[N - 1], fP[N - 1])}
    m, P = state_at[N - 1]
    for s, e in zip(reversed(starts), reversed(ends)):
        if s < e:
            E, g, Lc = chunk_smoother_aggregate(fm, fP, A, Pinf, H, y, R, s, e, Q)
            m, P = E @ m + g, E @ P @ E.T + Lc
        state_at[s] = (m, P)
    sm, sP = np.zeros((N, D), dtype), np.zeros((N, D, D), dtype)
    sm[N - 1], sP[N - 1] = state_at[N - 1]
    for s, e in zip(starts, ends):
        m, P = state_at[e]
        for k in range(e - 1, s - 1, -1):
            Pp = _pred(A[k + 1], fP[k], Pinf, None if Q is None else Q[k + 1])
            G = fP[k] @ A[k + 1].T @ np.linalg.inv(Pp)
            gk = fm[k] - G @ (A[k + 1] @ fm[k])
            Lk = fP[k] - G @ A[k + 1] @ fP[k]
            m, P = G @ m + gk, G @ P @ G.T + Lk
            sm[k], sP[k] = m, P
    return sm, sP, state_at


def sequential_posterior_mean(dt, kernel, y, R, dtype=np.float64, q_float64=False):
    """Sequential filter and RTS smoother with every array in `dtype`, returning
    the H-projected posterior means [N, P] (float64).  The predicted covariance is
    A (P - Pinf) A^T + Pinf (Q = Pinf - A Pinf A^T formed in `dtype`, as the
    float32 kernels did), or, with q_float64, A P A^T + Q with A and Q formed in
    float64 and rounded to `dtype` (q_float64 = "library": A and Q as the library's
    float32 kernels now form them)."""
    N = dt.shape[0]
    H = kernel.measurement_model().astype(dtype)
    Pinf64 = kernel.stationary_covariance()
    Pinf = Pinf64.astype(dtype)
    D = Pinf.shape[0]
    if q_float64 == "library":
        A, Q = _transitions(dt, kernel, dtype, "library")
    else:
        A64 = np.stack([kernel.state_transition(float(d)) for d in dt])
        A64[0] = np.eye(D)
        Q64 = Pinf64[None] - A64 @ Pinf64[None] @ np.swapaxes(A64, 1, 2)
        Q64[0] = 0.0
        A, Q = A64.astype(dtype), Q64.astype(dtype)
    y = y.reshape(N, -1).astype(dtype)
    R = R.reshape(N, y.shape[1], y.shape[1]).astype(dtype)

    def pred(k, P):
        return A[k] @ P @ A[k].T + Q[k] if q_float64 else A[k] @ (P - Pinf) @ A[k].T + Pinf

    m, P = np.zeros(D, dtype), Pinf.copy()
    fm, fP = np.zeros((N, D), dtype), np.zeros((N, D, D), dtype)
    for k in range(N):
        mp, Pp = A[k] @ m, pred(k, P)
        S = H @ Pp @ H.T + R[k]
        K = np.linalg.solve(S, H @ Pp).T
        m, P = mp + K @ (y[k] - H @ mp), Pp - K @ S @ K.T
        fm[k], fP[k] = m, P
    sm = fm.copy()
    for k in range(N - 2, -1, -1):
        Pp = pred(k + 1, fP[k])
        G = fP[k] @ A[k + 1].T @ np.linalg.inv(Pp)
        sm[k] = fm[k] + G @ (sm[k + 1] - A[k + 1] @ fm[k])
    return np.einsum("pd,nd->np", H.astype(np.float64), sm.astype(np.float64))
