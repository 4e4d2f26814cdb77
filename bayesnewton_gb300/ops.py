"""Filter / smoother operators (the interface of bayesnewton/ops.py:256-285 and
:357-380) and the prediction operator (bayesnewton/utils.py:123-138) on CUDA
tensors, computed by libbnx.so.

Arrays are torch CUDA tensors (numpy inputs are copied to the current device);
float32 or float64 selects the library's compiled precision.  Work is enqueued on
torch's current CUDA stream.
"""
import ctypes

import numpy as np
import torch

from . import _lib

_HANDLES = {}


def _tensor(x, dtype=None, device=None):
    if isinstance(x, torch.Tensor):
        t = x
    else:
        t = torch.as_tensor(np.asarray(x))
    if device is None:
        device = t.device if t.is_cuda else torch.device("cuda", torch.cuda.current_device())
    if dtype is None:
        dtype = t.dtype if t.dtype in (torch.float32, torch.float64) else torch.float64
    return t.to(device=device, dtype=dtype).contiguous()


def _dtype_code(dtype):
    if dtype == torch.float32:
        return _lib.DTYPE_F32
    if dtype == torch.float64:
        return _lib.DTYPE_F64
    raise TypeError("float32 or float64 expected, got %s" % dtype)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _handle(kernel, N, dtype):
    """A model handle for ops-level calls, cached by layout, length and dtype."""
    lib = _lib.load()
    desc = kernel.desc()
    key = (tuple(desc.size[:desc.num_components]), desc.combine, int(N), dtype,
           torch.cuda.current_device())
    h = _HANDLES.get(key)
    if h is None:
        lik = _lib.LikDesc()
        lik.kind = _lib.LIK_GAUSSIAN
        lik.variance = 1.0
        lik.num_cub = 20
        hp = ctypes.c_void_p()
        _lib.check(lib.bn_model_create(ctypes.byref(desc), ctypes.byref(lik), int(N), 1, _dtype_code(dtype), 0,
                                       ctypes.byref(hp)), "bn_model_create")
        h = hp
        _HANDLES[key] = h
    _lib.check(lib.bn_model_set_prior(h, ctypes.byref(desc)), "bn_model_set_prior")
    return h


def _result(h):
    lib = _lib.load()
    out = (ctypes.c_double * _lib.NRESULT)()
    st = ctypes.c_int32()
    _lib.check(lib.bn_model_result(h, _stream(), out, ctypes.byref(st)), "bn_model_result")
    return list(out), st.value


def kalman_filter(dt, kernel, y, noise_cov, mask=None, parallel=False, return_predict=False):
    """Run the Kalman filter over pseudo-observations y [N, P, 1] with covariances
    noise_cov [N, P, P] (mask [N, P] marks missing entries, excluded from the log
    marginal).  Returns (ell, (means [N, D, 1], covs [N, D, D])); with
    return_predict the one-step predictions are returned instead of the filtered
    states.  dt[0] is ignored: the first state is the stationary prior."""
    y = _tensor(y)
    dtype, dev = y.dtype, y.device
    N = y.shape[0]
    P = kernel.measurement_model().shape[0]
    D = kernel.state_dim
    y = y.reshape(N, P)
    dt = _tensor(dt, dtype, dev).reshape(N)
    R = _tensor(noise_cov, dtype, dev).reshape(N, P, P)
    m = None
    if mask is not None:
        m = _tensor(mask, torch.uint8, dev).reshape(N, P)
    means = torch.empty(N, D, 1, dtype=dtype, device=dev)
    covs = torch.empty(N, D, D, dtype=dtype, device=dev)
    h = _handle(kernel, N, dtype)
    lib = _lib.load()
    _lib.check(lib.bn_kalman_filter(h, _stream(), 1 if parallel else 0, 1 if return_predict else 0, _ptr(dt),
                                    _ptr(y), _ptr(R), _ptr(m), _ptr(means), _ptr(covs)), "bn_kalman_filter")
    res, _ = _result(h)
    return res[_lib.RES_LOGLIK], (means, covs)


def rauch_tung_striebel_smoother(dt, kernel, filter_mean, filter_cov, return_full=False, parallel=False):
    """RTS smoother from filtered means [N, D, 1] and covariances [N, D, D].  dt is
    the step from each time point to the next (the caller's shifted dt, as in
    basemodels.py:700).  Returns (means, covs, gains): H-projected [N, P, 1] and
    [N, P, P] unless return_full, and the gains [N, D, D].  The last time point's
    smoothed state is its filtered state."""
    fm = _tensor(filter_mean)
    dtype, dev = fm.dtype, fm.device
    N = fm.shape[0]
    D = kernel.state_dim
    P = kernel.measurement_model().shape[0]
    fm = fm.reshape(N, D)
    fP = _tensor(filter_cov, dtype, dev).reshape(N, D, D)
    dt = _tensor(dt, dtype, dev).reshape(N)
    k = D if return_full else P
    means = torch.empty(N, k, 1, dtype=dtype, device=dev)
    covs = torch.empty(N, k, k, dtype=dtype, device=dev)
    gains = torch.empty(N, D, D, dtype=dtype, device=dev)
    h = _handle(kernel, N, dtype)
    lib = _lib.load()
    _lib.check(lib.bn_rts_smoother(h, _stream(), 1 if parallel else 0, 1 if return_full else 0, _ptr(dt), _ptr(fm),
                                   _ptr(fP), _ptr(means), _ptr(covs), _ptr(gains)), "bn_rts_smoother")
    return means, covs, gains


def temporal_conditional(X, X_test, mean, cov, gain, kernel):
    """The state distribution at test times X_test from the smoothed states
    (mean [N, D, 1], cov [N, D, D]) and smoother gains [N, D, D] at the sorted
    training times (bayesnewton/utils.py:123-138).  X is the reference's augmented
    time vector [N + 2] with the dummy edge times -/+1e10 (the plain [N] training
    times are accepted too).  Returns (means [Nt, D, 1], covs [Nt, D, D])."""
    m = _tensor(mean)
    dtype, dev = m.dtype, m.device
    N = m.shape[0]
    D = kernel.state_dim
    x = _tensor(X, torch.float64, dev).reshape(-1)
    if x.shape[0] == N + 2:
        x = x[1:-1].contiguous()
    elif x.shape[0] != N:
        raise ValueError("X has %d times for %d states" % (x.shape[0], N))
    xt = _tensor(X_test, torch.float64, dev).reshape(-1)
    m = m.reshape(N, D)
    P = _tensor(cov, dtype, dev).reshape(N, D, D)
    G = _tensor(gain, dtype, dev).reshape(N, D, D)
    nt = xt.shape[0]
    means = torch.empty(nt, D, 1, dtype=dtype, device=dev)
    covs = torch.empty(nt, D, D, dtype=dtype, device=dev)
    h = _handle(kernel, N, dtype)
    lib = _lib.load()
    _lib.check(lib.bn_temporal_conditional(h, _stream(), _ptr(x), nt, _ptr(xt), _ptr(m), _ptr(P), _ptr(G), 1,
                                           _ptr(means), _ptr(covs)), "bn_temporal_conditional")
    return means, covs
