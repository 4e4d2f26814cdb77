"""One long series split into consecutive time segments, one per rank.

The parallel filter and smoother are associative scans, so a series can be cut
into G segments that run on G GPUs (one process each) with one small exchange
per scan: each rank scans its own segment, the G segment totals (one filter
element, d^2-sized, then one smoother element) are all-gathered, every rank
folds the totals of the segments before (after) it into the state entering
(leaving) its own segment, and finishes its scan locally.  The energy terms are
sums over time points, so one all-reduce of the result vector completes a step.

    seg = TimeSegment(kernel, likelihood, X, Y, rank, world)     # this rank's slice
    seg.inference(lr=1.0, exchange=TorchExchange())              # torch.distributed
    seg.energy()

Without torch.distributed, all segments can live in one process
(``run_segments``); that is how a single GPU checks the exchange against the
unsplit model.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .models import MarkovGaussianProcess, MarkovVariationalGP


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def fold_filter(totals, d):
    """Filtered state (m [d], P [d, d] flat) after the filter-element totals of
    the segments before this one, in order (an empty list: the series start)."""
    lib = _lib.load()
    state = None
    out = np.zeros(d + d * d)
    for t in totals:
        t = np.ascontiguousarray(t, dtype=np.float64)
        _lib.check(lib.bn_segment_filter_state(d, None if state is None else _dp(state), _dp(t), _dp(out)),
                   "bn_segment_filter_state")
        state = out.copy()
    return state


def fold_smoother(totals, d):
    """Smoothed state at the first step of the segment after this one, from the
    smoother-element totals of all later segments in time order (empty: none)."""
    lib = _lib.load()
    state = None
    out = np.zeros(d + d * d)
    for t in reversed(totals):
        t = np.ascontiguousarray(t, dtype=np.float64)
        _lib.check(lib.bn_segment_smoother_state(d, _dp(t), None if state is None else _dp(state), _dp(out)),
                   "bn_segment_smoother_state")
        state = out.copy()
    return state


class TorchExchange:
    """all_gather / all_reduce over the default torch.distributed group."""

    def __init__(self, device=None):
        self.device = device

    def gather(self, arr):
        import torch.distributed as dist
        dev = self.device if dist.get_backend() == "nccl" else torch.device("cpu")
        t = torch.as_tensor(arr, dtype=torch.float64, device=dev)
        out = [torch.empty_like(t) for _ in range(dist.get_world_size())]
        dist.all_gather(out, t)
        return [o.cpu().numpy() for o in out]

    def reduce_sum(self, arr):
        import torch.distributed as dist
        dev = self.device if dist.get_backend() == "nccl" else torch.device("cpu")
        t = torch.as_tensor(arr, dtype=torch.float64, device=dev)
        dist.all_reduce(t)
        return t.cpu().numpy()


def split_bounds(N, world):
    """[start, end) of each segment (equal counts, the remainder to the first ones)."""
    q, r = divmod(N, world)
    b = [0]
    for g in range(world):
        b.append(b[-1] + q + (1 if g < r else 0))
    return b


class TimeSegment:
    """Segment `rank` of `world` of the series (X, Y) (sorted inside), as a
    MarkovGaussianProcess over its own points (parallel form only)."""

    def __init__(self, kernel, likelihood, X, Y, rank, world, cls=MarkovVariationalGP, dtype=torch.float32,
                 device=None, **kw):
        X = np.asarray(X, dtype=np.float64).reshape(-1)
        Y = np.asarray(Y, dtype=np.float64)
        ind = np.argsort(X, kind="stable")
        X, Y = X[ind], Y[ind]
        b = split_bounds(X.shape[0], world)
        s, e = b[rank], b[rank + 1]
        if e <= s:
            raise ValueError("segment %d of %d is empty" % (rank, world))
        self.rank, self.world = rank, world
        self.model = cls(kernel, likelihood, X[s:e], Y[s:e], dtype=dtype, device=device, **kw)
        m = self.model
        dt = np.concatenate([[0.0], np.diff(X)])
        m.dt = torch.as_tensor(dt[s:e], device=m.device).to(dtype).contiguous()
        self.dt_next = float(X[e] - X[e - 1]) if e < X.shape[0] else 0.0
        _lib.check(m._lib.bn_model_set_segment(m._handle, 1 if rank > 0 else 0, 1 if e < X.shape[0] else 0,
                                               self.dt_next), "bn_model_set_segment")
        fe, se, stw = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        m._lib.bn_model_element_sizes(m._handle, ctypes.byref(fe), ctypes.byref(se), ctypes.byref(stw))
        self.fe, self.se, self.stw = fe.value, se.value, stw.value
        self.d = m.state_dim
        self.result = None

    def _phase(self, phase, newton, lr, boundary):
        m = self.model
        total = np.zeros(max(self.fe, self.se)) if phase < 2 else None
        _lib.check(m._lib.bn_segment_step(m._handle, m._stream(), phase, 1 if newton else 0, float(lr),
                                          m.dt.data_ptr(), m.Y.data_ptr(), ctypes.byref(m._state),
                                          None if boundary is None else _dp(boundary),
                                          None if total is None else _dp(total)), "bn_segment_step")
        if phase == 0:
            return total[:self.fe].copy()
        if phase == 1:
            return total[:self.se].copy()
        return None

    def step_phases(self, newton, lr, gather):
        """Phases 0-2 with `gather(local_total) -> [total of every segment]`."""
        tf = gather(self._phase(0, newton, lr, None))
        left = fold_filter(tf[:self.rank], self.d)
        ts = gather(self._phase(1, newton, lr, left))
        right = fold_smoother(ts[self.rank + 1:], self.d)
        self._phase(2, newton, lr, right)
        self.model._result = None
        res, status = self.model._fetch()
        return np.asarray(res, dtype=np.float64), status

    def inference(self, lr=1.0, exchange=None):
        exchange = exchange or TorchExchange(self.model.device)
        if self.result is None:  # the posterior of the initial sites, as inference() does
            self._finish(self.step_phases(False, 1.0, exchange.gather), exchange)
        self._finish(self.step_phases(True, lr, exchange.gather), exchange)

    def _finish(self, rs, exchange):
        res, status = rs
        self.result = exchange.reduce_sum(res)
        self.status = status

    def energy(self):
        return float(self.result[_lib.RES_ENERGY])


def run_segments(segments, newton, lr):
    """Step all segments of one series held in this process (phases in lockstep,
    the exchange done in memory).  Returns the summed result vector."""
    tf = [s._phase(0, newton, lr, None) for s in segments]
    ts = []
    for s in segments:
        ts.append(s._phase(1, newton, lr, fold_filter(tf[:s.rank], s.d)))
    tot = None
    for s in segments:
        s._phase(2, newton, lr, fold_smoother(ts[s.rank + 1:], s.d))
        s.model._result = None
        r = np.asarray(s.model._fetch()[0], dtype=np.float64)
        tot = r if tot is None else tot + r
    return tot
