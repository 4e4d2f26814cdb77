"""Oracle Kalman filter and RTS smoother (float64 numpy restatement).

Follows bayesnewton/ops.py:
  process_noise_covariance (:149-151), _sequential_kf (:154-180),
  parallel_filtering_element_ / operator / make_associative_filtering_elements
  (:183-229), _parallel_kf (:237-253), kalman_filter (:256-285),
  _sequential_rts (:288-311), parallel smoothing element / operator / _parallel_rts
  (:314-354), rauch_tung_striebel_smoother (:357-380);
and bayesnewton/utils.py: mvn_logpdf (:376-396), predict_from_state (:99-118),
temporal_conditional (:123-138), compute_conditional_statistics (:172-213).

The associative scan is the odd/even recursion that jax.lax.associative_scan uses
(jax 0.4.14, not vendored in the reference): combine adjacent pairs, recurse on
the pair results, then fix up the even positions.  Elements are tuples of arrays
with a leading sequence axis, so every level is one batched numpy expression.
"""
import math

import numpy as np

LOG2PI = math.log(2 * math.pi)
INV2PI = (2 * math.pi) ** -1


def T(P):
    return np.swapaxes(P, -1, -2)


def solve(P, Q):
    """P^-1 Q for PSD P via Cholesky (utils.py:14-19); batched over leading axes."""
    L = np.linalg.cholesky(P)
    Z = np.linalg.solve(L, Q)
    return np.linalg.solve(T(L), Z)


def inv(P):
    return solve(P, np.broadcast_to(np.eye(P.shape[-1]), P.shape).copy())


def mvn_logpdf(x, mean, cov, mask=None):
    """Masked Gaussian log density of one site (utils.py:376-396)."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, 1)
    mean = np.asarray(mean, dtype=np.float64).reshape(-1, 1)
    cov = np.array(cov, dtype=np.float64)
    if mask is not None:
        maskv = np.asarray(mask, dtype=bool).reshape(-1, 1)
        x = np.where(maskv, 0.0, x)
        mean = np.where(maskv, 0.0, mean)
        cov = np.where(maskv | maskv.T, 0.0, cov)
        cov = np.where(np.diag(maskv[:, 0]), INV2PI, cov)
    n = mean.shape[0]
    L = np.linalg.cholesky(cov)
    log_det = 2 * np.sum(np.log(np.abs(np.diag(L))))
    diff = x - mean
    z = np.linalg.solve(L, diff)
    return float(-0.5 * ((z.T @ z).item() + n * LOG2PI + log_det))


def mvn_logpdf_batched(x, mean, cov, mask=None):
    """vmap of mvn_logpdf over a leading axis (ops.py:232-234)."""
    out = np.empty(x.shape[0])
    for i in range(x.shape[0]):
        out[i] = mvn_logpdf(x[i], mean[i], cov[i], None if mask is None else mask[i])
    return out


def process_noise_covariance(A, Pinf):
    return Pinf - A @ Pinf @ T(A)


def discretise(dt, kernel):
    Pinf = kernel.stationary_covariance()
    As = np.atleast_3d(kernel.state_transition(np.atleast_1d(dt)))
    if As.ndim == 2:
        As = As[:, None, None]
    Qs = process_noise_covariance(As, Pinf)
    return As, Qs, kernel.measurement_model(), Pinf


# ----------------------------------------------------------------------------- filter

def _sequential_kf(As, Qs, H, ys, noise_covs, m0, P0, masks, return_predict=False):
    N = As.shape[0]
    d = m0.shape[0]
    m, P, ell = m0, P0, 0.0
    fms = np.empty([N, d, 1])
    fPs = np.empty([N, d, d])
    for n in range(N):
        A, Q, y, R = As[n], Qs[n], ys[n], noise_covs[n]
        m_ = A @ m
        P_ = A @ P @ A.T + Q
        obs_mean = H @ m_
        HP = H @ P_
        S = HP @ H.T + R
        ell += mvn_logpdf(y, obs_mean, S, None if masks is None else masks[n])
        K = solve(S, HP).T
        m = m_ + K @ (y - obs_mean)
        P = P_ - K @ HP
        if return_predict:
            fms[n], fPs[n] = m_, P_
        else:
            fms[n], fPs[n] = m, P
    return ell, fms, fPs


def parallel_filtering_element(A, Q, H, R, y):
    """ops.py:183-197, batched over the leading axis."""
    HQ, HA = H @ Q, H @ A
    S = HQ @ T(H) + R
    SinvH = solve(S, np.broadcast_to(H, S.shape[:-1] + (H.shape[-1],)).copy())
    K = Q @ T(SinvH)
    AA = A - K @ HA
    b = K @ y
    C = Q - K @ HQ
    SinvHA = T(SinvH @ A)
    eta = SinvHA @ y
    J = SinvHA @ HA
    return AA, b, C, J, eta


def parallel_filtering_operator(elem1, elem2):
    """ops.py:203-219 (inverts C1 as the reference does)."""
    A1, b1, C1, J1, eta1 = elem1
    A2, b2, C2, J2, eta2 = elem2
    C1inv = inv(C1)
    temp = solve(C1inv + J2, C1inv)
    A2temp = A2 @ temp
    AA = A2temp @ A1
    b = A2temp @ (b1 + C1 @ eta2) + b2
    C = A2temp @ C1 @ T(A2) + C2
    A1temp = T(A1) @ T(temp)
    eta = A1temp @ (eta2 - J2 @ b1) + eta1
    J = A1temp @ J2 @ A1 + J1
    return AA, b, C, J, eta


def parallel_filtering_operator_stable(elem1, elem2):
    """The same combine written with (I + C1 J2)^-1, which also holds when C1 is
    singular (Sarkka & Garcia-Fernandez 2021, eq. 16)."""
    A1, b1, C1, J1, eta1 = elem1
    A2, b2, C2, J2, eta2 = elem2
    d = A1.shape[-1]
    W = np.linalg.inv(np.eye(d) + C1 @ J2)
    A2W = A2 @ W
    AA = A2W @ A1
    b = A2W @ (b1 + C1 @ eta2) + b2
    C = A2W @ C1 @ T(A2) + C2
    A1W = T(A1) @ T(W)
    eta = A1W @ (eta2 - J2 @ b1) + eta1
    J = A1W @ J2 @ A1 + J1
    return AA, b, C, J, eta


def associative_scan(fn, elems, reverse=False):
    """Inclusive scan with the odd/even recursion of jax.lax.associative_scan."""
    elems = [np.asarray(e) for e in elems]
    if reverse:
        elems = [e[::-1] for e in elems]

    def _scan(es):
        n = es[0].shape[0]
        if n < 2:
            return es
        reduced = fn([e[0:-1:2] for e in es], [e[1::2] for e in es])
        odd = _scan(list(reduced))
        if n % 2 == 0:
            even = fn([e[:-1] for e in odd], [e[2::2] for e in es])
        else:
            even = fn(odd, [e[2::2] for e in es])
        even = [np.concatenate([e[0:1], r]) for e, r in zip(es, even)]
        out = []
        for ev, od in zip(even, odd):
            o = np.empty((n,) + ev.shape[1:], dtype=ev.dtype)
            o[0::2] = ev
            o[1::2] = od
            out.append(o)
        return out

    res = _scan(elems)
    if reverse:
        res = [r[::-1] for r in res]
    return res


def make_associative_filtering_elements(As, Qs, H, ys, noise_covs, m0, P0):
    """ops.py:222-229."""
    Qs = Qs.copy()
    Qs[0] = P0
    AA, b, C, J, eta = parallel_filtering_element(As, Qs, H, noise_covs, ys)
    S = H @ Qs[0] @ H.T + noise_covs[0]
    K0 = solve(S, H @ Qs[0]).T
    b = b.copy()
    b[0] += m0 - K0 @ H @ m0
    return AA, b, C, J, eta


def _parallel_kf(As, Qs, H, ys, noise_covs, m0, P0, masks, return_predict=False, stable=False):
    """ops.py:237-253."""
    elems = make_associative_filtering_elements(As, Qs, H, ys, noise_covs, m0, P0)
    op = parallel_filtering_operator_stable if stable else parallel_filtering_operator
    final = associative_scan(op, elems)
    fms, fPs = final[1], final[2]
    mpred = As @ np.concatenate([m0[None], fms[:-1]])
    Ppred = As @ np.concatenate([P0[None], fPs[:-1]]) @ T(As) + Qs
    loglik = np.sum(mvn_logpdf_batched(ys, H @ mpred, H @ Ppred @ H.T + noise_covs, masks))
    if return_predict:
        return loglik, mpred, Ppred
    return loglik, fms, fPs


def kalman_filter(dt, kernel, y, noise_cov, mask=None, parallel=False, return_predict=False,
                  stable=False):
    """ops.py:256-285: returns (ell, (means [N,d,1], covs [N,d,d]))."""
    y = np.asarray(y, dtype=np.float64)
    noise_cov = np.asarray(noise_cov, dtype=np.float64)
    if mask is None:
        mask = np.zeros(y.shape[:2], dtype=bool)
    As, Qs, H, Pinf = discretise(dt, kernel)
    minf = np.zeros([Pinf.shape[0], 1])
    if parallel:
        ell, m, P = _parallel_kf(As, Qs, H, y, noise_cov, minf, Pinf, mask, return_predict, stable)
    else:
        ell, m, P = _sequential_kf(As, Qs, H, y, noise_cov, minf, Pinf, mask, return_predict)
    return ell, (m, P)


# ----------------------------------------------------------------------------- smoother

def _sequential_rts(fms, fPs, As, Qs, H, return_full):
    """ops.py:288-311 (reverse scan; the carry starts at the last filter state)."""
    N, d = fms.shape[0], fms.shape[1]
    sm, sP = fms[-1], fPs[-1]
    p = H.shape[0]
    sms = np.empty([N, d if return_full else p, 1])
    sPs = np.empty([N] + ([d, d] if return_full else [p, p]))
    gains = np.empty([N, d, d])
    for n in range(N - 1, -1, -1):
        fm, fP, A, Q = fms[n], fPs[n], As[n], Qs[n]
        pm = A @ fm
        AfP = A @ fP
        pP = AfP @ A.T + Q
        C = solve(pP, AfP).T
        sm = fm + C @ (sm - pm)
        sP = fP + C @ (sP - pP) @ C.T
        if return_full:
            sms[n], sPs[n] = sm, sP
        else:
            sms[n], sPs[n] = H @ sm, H @ sP @ H.T
        gains[n] = C
    return sms, sPs, gains


def parallel_smoothing_element(A, Q, m, P):
    """ops.py:318-325."""
    Pp = A @ P @ T(A) + Q
    E = T(solve(Pp, A @ P))
    g = m - E @ A @ m
    L = P - E @ Pp @ T(E)
    return E, g, L


def parallel_smoothing_operator(elem1, elem2):
    """ops.py:328-335."""
    E1, g1, L1 = elem1
    E2, g2, L2 = elem2
    return E2 @ E1, E2 @ g1 + g2, E2 @ L1 @ T(E2) + L2


def _parallel_rts(fms, fPs, As, Qs, H, return_full):
    """ops.py:338-354."""
    E, g, L = parallel_smoothing_element(As, Qs, fms, fPs)
    gains = E
    E = np.concatenate([E[:-1], np.zeros_like(fPs[-1])[None]])
    g = np.concatenate([g[:-1], fms[-1][None]])
    L = np.concatenate([L[:-1], fPs[-1][None]])
    final = associative_scan(parallel_smoothing_operator, [E, g, L], reverse=True)
    sms, sPs = final[1], final[2]
    if return_full:
        return sms, sPs, gains
    return H @ sms, H @ sPs @ H.T, gains


def rauch_tung_striebel_smoother(dt, kernel, filter_mean, filter_cov, return_full=False,
                                 parallel=False):
    """ops.py:357-380."""
    As, Qs, H, _ = discretise(dt, kernel)
    if parallel:
        return _parallel_rts(filter_mean, filter_cov, As, Qs, H, return_full)
    return _sequential_rts(filter_mean, filter_cov, As, Qs, H, return_full)


# ----------------------------------------------------------------------------- prediction

def compute_conditional_statistics(x_test, x, kernel, ind):
    """utils.py:172-213: P = [A_fwd - W A_back A_fwd, W], T for every test time,
    with W = Q_fwd A_back^T Q_mp^-1 and Q_mp = Q_back + A_back Q_fwd A_back^T
    (the 1e-8 jitter added before the Cholesky solve)."""
    dt_fwd = x_test - x[ind]
    dt_back = x[ind + 1] - x_test
    A_fwd, Q_fwd, _, _ = discretise(dt_fwd, kernel)
    A_back, Q_back, _, _ = discretise(dt_back, kernel)
    A_back_Q_fwd = A_back @ Q_fwd
    Q_mp = Q_back + A_back @ T(A_back_Q_fwd)
    jitter = 1e-8 * np.eye(Q_mp.shape[-1])
    Q_mp_inv_A_back = solve(Q_mp + jitter, A_back)
    Tc = Q_fwd - T(A_back_Q_fwd) @ Q_mp_inv_A_back @ Q_fwd
    W = Q_fwd @ T(Q_mp_inv_A_back)
    P = np.concatenate([A_fwd - W @ A_back @ A_fwd, W], axis=-1)
    return P, Tc


def predict_from_state(x_test, ind, x, post_mean, post_cov, gain, kernel):
    """utils.py:99-118 (vectorised over the test times): the state at each test
    time given the joint smoothed posterior of its two neighbouring states."""
    P, Tc = compute_conditional_statistics(x_test, x, kernel, ind)
    mean_joint = np.concatenate([post_mean[ind], post_mean[ind + 1]], axis=1)
    cross = gain[ind] @ post_cov[ind + 1]
    cov_joint = np.concatenate([np.concatenate([post_cov[ind], cross], axis=2),
                                np.concatenate([T(cross), post_cov[ind + 1]], axis=2)], axis=1)
    return P @ mean_joint, P @ cov_joint @ T(P) + Tc


def temporal_conditional(X, X_test, mean, cov, gain, kernel):
    """utils.py:123-138: X holds the training times with a dummy state at each
    edge (prior mean 0, covariance Pinf, gain 0 before the first)."""
    Pinf = kernel.stationary_covariance()[None, ...]
    minf = np.zeros([1, Pinf.shape[1], 1])
    mean_aug = np.concatenate([minf, mean, minf])
    cov_aug = np.concatenate([Pinf, cov, Pinf])
    gain = np.concatenate([np.zeros_like(gain[:1]), gain])
    x = np.asarray(X, dtype=np.float64).reshape(-1)
    xt = np.asarray(X_test, dtype=np.float64).reshape(-1)
    ind_test = np.searchsorted(x, xt) - 1
    return predict_from_state(xt, ind_test, x, mean_aug, cov_aug, gain, kernel)


# ----------------------------------------------------------------------------- infinite horizon

def dare(A, H, Q, R, Pinit, num_iters=20):
    """ops.py:796-822: num_iters steps of the Riccati recursion from Pinit."""
    X = Pinit
    for _ in range(num_iters):
        HX = H @ X
        S = HX @ H.T + R
        K = solve(S, HX).T
        X = A @ (X - K @ HX) @ A.T + Q
    return X


def _sequential_kf_ih(AKHAs, HA, Kys, Ss, ys, m0, masks):
    """ops.py:825-845."""
    m, ell = m0, 0.0
    fms = np.empty([ys.shape[0]] + list(m0.shape))
    for n in range(ys.shape[0]):
        ell += mvn_logpdf(ys[n], HA @ m, Ss[n], masks[n])
        m = AKHAs[n] @ m + Kys[n]
        fms[n] = m
    return ell, fms


def _parallel_kf_ih(AKHAs_or_iAKHAs, HA, Kys, Ss, ys, m0, masks, heteroscedastic):
    """ops.py:848-877: associative scan of (B, v); the heteroscedastic operator takes
    the inverse transition matrices and solves with them (ops.py:855-859)."""
    if heteroscedastic:
        def op(e1, e2):
            B1, v1 = e1
            B2, v2 = e2
            return B1 @ B2, np.linalg.solve(B2, v1) + v2
    else:
        def op(e1, e2):
            B1, v1 = e1
            B2, v2 = e2
            return B1 @ B2, B2 @ v1 + v2
    fms = associative_scan(op, [AKHAs_or_iAKHAs, Kys])[1]
    obs_means = HA @ np.concatenate([m0[None], fms[:-1]])
    ell = 0.0
    for n in range(ys.shape[0]):
        ell += mvn_logpdf(ys[n], obs_means[n], Ss[n], masks[n])
    return ell, fms


def kalman_filter_infinite_horizon(dt, kernel, y, noise_cov, mask=None, parallel=False, heteroscedastic=False,
                                   noise_cov_tied=None, dare_iters=20, dare_init=None):
    """ops.py:880-955: steady-state covariance by the warm-started DARE with the tied
    noise; per-site gains when heteroscedastic.  Returns (ell, (means, (Pdare, cov)))."""
    N = y.shape[0]
    if mask is None:
        mask = np.zeros(y.shape[:2], dtype=bool)
    Pinf = kernel.stationary_covariance()
    minf = np.zeros([Pinf.shape[0], 1])
    A = np.atleast_3d(kernel.state_transition(np.atleast_1d(dt[1])))[0]
    Q = Pinf - A @ Pinf @ A.T
    H = kernel.measurement_model()
    Pdare = dare(A, H, Q, noise_cov_tied, Pinf if dare_init is None else dare_init, dare_iters)
    S = H @ Pdare @ H.T + noise_cov_tied
    K = Pdare @ solve(S, H).T
    HA = H @ A
    if heteroscedastic:
        Ss = H @ Pdare @ H.T + noise_cov
        Ks = Pdare @ T(np.linalg.solve(Ss, np.tile(H, [N, 1, 1])))
        AKHAs = A - Ks @ HA
    else:
        Ss = np.tile(S, [N, 1, 1])
        Ks = np.tile(K, [N, 1, 1])
        AKHAs = np.tile(A - K @ HA, [N, 1, 1])
    Kys = Ks @ y
    cov = Pdare - K @ H @ Pdare
    masks = [None if not np.any(mask[n]) else mask[n] for n in range(N)]
    if parallel:
        if heteroscedastic:
            iA = np.atleast_3d(kernel.state_transition(np.atleast_1d(-dt[1])))[0]
            iAKHAs = iA + iA @ ((Pdare @ H.T) @ np.linalg.solve(noise_cov, np.tile(H, [N, 1, 1])))
            ell, means = _parallel_kf_ih(iAKHAs, HA, Kys, Ss, y, minf, masks, True)
        else:
            ell, means = _parallel_kf_ih(AKHAs, HA, Kys, Ss, y, minf, masks, False)
    else:
        ell, means = _sequential_kf_ih(AKHAs, HA, Kys, Ss, y, minf, masks)
    return ell, (means, (Pdare, cov))


def rts_dare(A, Q, Pinf, num_iters=20):
    """ops.py:958-975."""
    X = Pinf
    for _ in range(num_iters):
        X = A @ X @ A.T + Q
    return X


def rauch_tung_striebel_smoother_infinite_horizon(dt, kernel, filter_mean, filter_cov, return_full=False,
                                                  parallel=False, dare_iters=20, dare_init=None):
    """ops.py:1018-1068 (sequential form :978-993; the parallel form :1003-1015 runs
    the same affine recursion as a reverse associative scan)."""
    Pinf = kernel.stationary_covariance()
    A = np.atleast_3d(kernel.state_transition(np.atleast_1d(dt[0])))[0]
    H = kernel.measurement_model()
    N = dt.shape[0]
    Pdare, fcov = filter_cov
    gain = fcov @ solve(Pdare, A).T
    Qdare = fcov - gain @ Pdare @ gain.T
    dare_cov = rts_dare(gain, Qdare, Pinf if dare_init is None else dare_init, dare_iters)
    Afms = A @ filter_mean
    if parallel:
        gains = np.tile(gain, [N, 1, 1])
        E = np.concatenate([gains, np.zeros_like(gain)[None]])
        g = np.concatenate([filter_mean - gains @ Afms, filter_mean[-1][None]])

        def op(e1, e2):
            B1, v1 = e1
            B2, v2 = e2
            return B1 @ B2, B2 @ v1 + v2
        sms = associative_scan(op, [E, g], reverse=True)[1][:-1]
    else:
        sms = np.empty_like(filter_mean)
        sm = filter_mean[-1]
        for n in range(N - 1, -1, -1):
            sm = filter_mean[n] + gain @ (sm - Afms[n])
            sms[n] = sm
    means = sms if return_full else H @ sms
    cov = dare_cov if return_full else H @ dare_cov @ H.T
    return means, np.tile(cov, [N, 1, 1]), np.tile(gain, [N, 1, 1]), dare_cov


# ----------------------------------------------------------------------------- mean field

def _block_project(P, sizes):
    """Zero the cross-block entries (the mean-field block-diagonal covariance)."""
    out = np.zeros_like(P)
    o = 0
    for s in sizes:
        out[..., o:o + s, o:o + s] = P[..., o:o + s, o:o + s]
        o += s
    return out


def kalman_filter_meanfield(dt, kernel, y, noise_cov, mask=None, block_sizes=None):
    """_sequential_kf_mf (ops.py:429-463) with kalman_filter_meanfield (:580-604): the
    filter of the independent latents with the covariance kept block-diagonal after
    every predict and update."""
    As, Qs, H, Pinf = discretise(dt, kernel)
    m = np.zeros([Pinf.shape[0], 1])
    P = Pinf
    N = y.shape[0]
    ell = 0.0
    fms = np.empty([N, Pinf.shape[0], 1])
    fPs = np.empty([N] + list(Pinf.shape))
    for n in range(N):
        m = As[n] @ m
        P = _block_project(As[n] @ P @ As[n].T + Qs[n], block_sizes)
        HP = H @ P
        S = HP @ H.T + noise_cov[n]
        ell += mvn_logpdf(y[n], H @ m, S, None if mask is None else mask[n])
        K = solve(S, HP).T
        m = m + K @ (y[n] - H @ m)
        P = _block_project(P - K @ HP, block_sizes)
        fms[n], fPs[n] = m, P
    return ell, (fms, fPs)


def rauch_tung_striebel_smoother_meanfield(dt, kernel, filter_mean, filter_cov, block_sizes=None):
    """_sequential_rts_mf (ops.py:617-644) with rauch_tung_striebel_smoother_meanfield
    (:674-706): the RTS recursion on the block-diagonal covariances; H-projected."""
    As, Qs, H, _ = discretise(dt, kernel)
    N = filter_mean.shape[0]
    sm, sP = filter_mean[-1], filter_cov[-1]
    sms = np.empty([N, H.shape[0], 1])
    sPs = np.empty([N, H.shape[0], H.shape[0]])
    for n in range(N - 1, -1, -1):
        fm, fP, A, Q = filter_mean[n], filter_cov[n], As[n], Qs[n]
        pm = A @ fm
        AfP = A @ fP
        pP = AfP @ A.T + Q
        C = solve(pP, AfP).T
        sm = fm + C @ (sm - pm)
        sP = fP + C @ (sP - pP) @ C.T
        sms[n], sPs[n] = H @ sm, H @ _block_project(sP, block_sizes) @ H.T
    return sms, sPs
