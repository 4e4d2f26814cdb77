"""Many independent Markov GPs stepped together.

The reference fits one series per model object, so a collection of series costs
one filter/smoother pass (and, on a GPU backend, one set of launches) per series.
Here the series are concatenated into one time axis of sum(N_i) steps and one
inference step runs them all: a series start is a transition with A = 0 (the
state restarts from the series' stationary prior), so the chunked associative
scan runs across series boundaries unchanged, and each chunk reads its series'
hyperparameters from a per-series table.

    batch = MarkovSeriesBatch([(Matern32(v, l), Gaussian(0.05), X, Y), ...])
    batch.inference(lr=1.0)          # all series: site update + filter + smoother
    batch.series_energy()            # energy of each series (numpy array)

Every series uses the same kernel family (a single Matern12/32/52/72, whose
variance and lengthscale may differ per series) and the same inference method
(VI or Newton); the likelihood may differ per series (Gaussian with its own
noise, Poisson with exp link, Bernoulli).  Each series' results equal those of
the corresponding single-series MarkovGaussianProcess.
"""
import ctypes
import json
import os

import numpy as np
import torch

from . import _lib
from .cubature import GaussHermite
from .kernels import Matern12, Matern32, Matern52, Matern72
from .likelihoods import Bernoulli, Gaussian, Poisson
from .models import MarkovGaussianProcess

_SINGLE = (Matern12, Matern32, Matern52, Matern72)


def autotune_key(device_name, kernel_family, num_series, num_data, dtype, method):
    """Key of an autotuned chunk length in the cache file: the choice depends on
    the GPU, the kernel family (state size), the batch's shape, dtype and method."""
    return "%s|%s|S=%d|N=%d|%s|%s" % (device_name, kernel_family, int(num_series), int(num_data),
                                     str(dtype).replace("torch.", ""), method)


def load_autotune_cache(path):
    """{key: {"steps_per_thread": L, "ms": {L: ms}}} from a JSON cache file ({} if
    the file does not exist)."""
    if not path or not os.path.exists(path):
        return {}
    with open(path) as f:
        data = json.load(f)
    if not isinstance(data, dict):
        raise ValueError("autotune cache %s does not hold a JSON object" % path)
    return data


def store_autotune_cache(path, key, steps_per_thread, times):
    """Add (or replace) one entry and rewrite the file atomically."""
    data = load_autotune_cache(path)
    data[key] = {"steps_per_thread": int(steps_per_thread), "ms": {str(k): float(v) for k, v in times.items()}}
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


class MarkovSeriesBatch(MarkovGaussianProcess):
    """Independent series [(kernel, likelihood, X, Y), ...] on one device.

    steps_per_thread: scan chunk length; 0 picks it from the total length, and
    autotune=True times the candidate lengths on the data and keeps the fastest
    (autotune="path.json" also reads and writes that cache file, see autotune()).
    """
    _method = _lib.METHOD_VI

    def __init__(self, series, method="vi", dtype=torch.float32, device=None, cubature=None, steps_per_thread=0,
                 autotune=False, score_form=None):
        if not series:
            raise ValueError("no series")
        kcls = type(series[0][0])
        if kcls not in _SINGLE:
            raise NotImplementedError("batched series need a single Matern kernel, got %s" % kcls.__name__)
        for k, lik, _, _ in series:
            if type(k) is not kcls:
                raise ValueError("every series must use the same kernel family")
            if not isinstance(lik, (Gaussian, Poisson, Bernoulli)):
                raise NotImplementedError("batched series need a single-latent likelihood")
        bins = {float(lik.binsize) for _, lik, _, _ in series if isinstance(lik, Poisson)}
        if len(bins) > 1:
            raise ValueError("Poisson series must share one binsize")
        self._method = {"vi": _lib.METHOD_VI, "newton": _lib.METHOD_NEWTON}[method]
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        dev = torch.device(device)
        # concatenate the series, each sorted in time with dt = 0 at its start
        xs, ys, dts, offsets = [], [], [], [0]
        for _, _, X, Y in series:
            x = np.asarray(X, dtype=np.float64).reshape(-1)
            y = np.asarray(Y, dtype=np.float64).reshape(-1)
            if x.shape[0] != y.shape[0] or x.shape[0] < 1:
                raise ValueError("each series needs as many inputs as outputs, at least one")
            ind = np.argsort(x, kind="stable")
            x, y = x[ind], y[ind]
            xs.append(x)
            ys.append(y)
            dts.append(np.concatenate([[0.0], np.diff(x)]))
            offsets.append(offsets[-1] + x.shape[0])
        self.series = series
        self.num_series = len(series)
        self.offsets = np.asarray(offsets, dtype=np.int64)
        X = np.concatenate(xs)
        Y = np.concatenate(ys)
        # the representative likelihood carries the shared settings (cubature,
        # Poisson binsize); each series' kind and noise come from its own
        rep = next((lik for _, lik, _, _ in series if isinstance(lik, Poisson)), series[0][1])
        super().__init__(series[0][0], rep, X[:, None], Y[:, None], parallel=True, dtype=dtype, device=dev,
                         cubature=cubature or GaussHermite(), steps_per_thread=steps_per_thread,
                         score_form=score_form)
        # input_admin sorted the concatenation by time: restore the series order
        self.X = torch.as_tensor(X, device=dev).to(dtype)[:, None].contiguous()
        self.Y = torch.as_tensor(Y, device=dev).to(dtype)[:, None].contiguous()
        self.dt = torch.as_tensor(np.concatenate(dts), device=dev).to(dtype).contiguous()
        self._tables = self._series_tables()
        self._set_series(self._handle)
        self._ser_versions = self._series_versions()
        self.steps_per_thread = self.chunking()[0]
        if autotune:
            self.autotune(cache=autotune if isinstance(autotune, str) else None)

    # ------------------------------------------------------------ per-series tables
    def _series_versions(self):
        return tuple((k.version, lik.version) for k, lik, _, _ in self.series)

    def _series_tables(self):
        var = np.array([k.variance for k, _, _, _ in self.series], dtype=np.float64)
        ell = np.array([k.lengthscale for k, _, _, _ in self.series], dtype=np.float64)
        kind = np.array([lik.kind() for _, lik, _, _ in self.series], dtype=np.int32)
        lvar = np.array([float(getattr(lik, "variance", 1.0)) for _, lik, _, _ in self.series], dtype=np.float64)
        return var, ell, kind, lvar

    def _set_series(self, handle):
        var, ell, kind, lvar = self._tables
        dp = ctypes.POINTER(ctypes.c_double)
        _lib.check(self._lib.bn_model_set_series(
            handle, self.num_series, self.offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            var.ctypes.data_as(dp), ell.ctypes.data_as(dp), kind.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            lvar.ctypes.data_as(dp)), "bn_model_set_series")

    def _sync_params(self):
        v = self._series_versions()
        if v != self._ser_versions:
            self._tables = self._series_tables()
            self._set_series(self._handle)
            self._ser_versions = v
            self._stale = True

    # ------------------------------------------------------------ results
    def series_energy(self):
        """Energy of each series at the current posterior (numpy [num_series])."""
        self._sync_params()
        if self._stale:
            self.update_posterior()
        out = np.zeros(self.num_series, dtype=np.float64)
        _lib.check(self._lib.bn_model_series_energy(self._handle, self._stream(),
                                                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
                   "bn_model_series_energy")
        return out

    def series_slice(self, i):
        return slice(int(self.offsets[i]), int(self.offsets[i + 1]))

    def series_posterior(self, i):
        """(mean [N_i], variance [N_i]) of series i."""
        sl = self.series_slice(i)
        return self._pm[sl, 0], self._pv[sl, 0, 0]

    # ------------------------------------------------------------ autotuner
    def _state_tensors(self):
        return (self._nat1, self._nat2, self._pm, self._pv, self._grad, self._hess, self._lin)

    def autotune_key(self):
        name = torch.cuda.get_device_name(self.device)
        method = {_lib.METHOD_VI: "vi", _lib.METHOD_NEWTON: "newton"}[self._method]
        return autotune_key(name, type(self.kernel).__name__, self.num_series, self.num_data, self.dtype, method)

    def _use_chunk_length(self, L):
        """Replace the model handle by one with chunk length L."""
        code = {torch.float32: _lib.DTYPE_F32, torch.float64: _lib.DTYPE_F64}[self.dtype]
        h = ctypes.c_void_p()
        _lib.check(self._lib.bn_model_create(ctypes.byref(self.kernel.desc()), ctypes.byref(self._lik_desc()),
                                             self.num_data, self.obs_dim, code, int(L), ctypes.byref(h)),
                   "bn_model_create")
        self._set_series(h)
        self._lib.bn_model_destroy(self._handle)
        self._handle = h
        self.steps_per_thread = int(L)
        self._result = None

    def autotune(self, candidates=(4, 8, 16, 32, 64), reps=5, cache=None):
        """Time one Newton step per candidate chunk length (CUDA events on the
        current stream, the model state restored after each trial) and keep the
        fastest.  Returns {steps_per_thread: ms}.

        cache: path of a JSON file of earlier choices keyed by GPU name, kernel
        family, number of series, total length, dtype and method.  A stored
        choice is used without timing (the returned times are the stored ones);
        otherwise the timed choice is added to the file."""
        if cache:
            entry = load_autotune_cache(cache).get(self.autotune_key())
            if entry is not None:
                # as after timing: the current posterior computed, then the chosen handle
                self._sync_params()
                if self._stale:
                    self.update_posterior()
                self._use_chunk_length(entry["steps_per_thread"])
                return {int(k): float(v) for k, v in entry["ms"].items()}
        times = self._autotune_timed(candidates, reps)
        if cache:
            store_autotune_cache(cache, self.autotune_key(), self.steps_per_thread, times)
        return times

    def _autotune_timed(self, candidates, reps):
        self._sync_params()
        if self._stale:
            self.update_posterior()
        saved = [t.clone() for t in self._state_tensors()]
        code = {torch.float32: _lib.DTYPE_F32, torch.float64: _lib.DTYPE_F64}[self.dtype]
        stream = torch.cuda.current_stream(self.device)
        times = {}
        best = (float("inf"), None, None)
        for L in candidates:
            if L * 2 > self.num_data and L != candidates[0]:
                continue
            h = ctypes.c_void_p()
            _lib.check(self._lib.bn_model_create(ctypes.byref(self.kernel.desc()), ctypes.byref(self._lik_desc()),
                                                 self.num_data, self.obs_dim, code, int(L), ctypes.byref(h)),
                       "bn_model_create")
            self._set_series(h)
            step = lambda: _lib.check(self._lib.bn_newton_step(h, self._stream(), 1, 1.0, self.dt.data_ptr(),
                                                               self.Y.data_ptr(), ctypes.byref(self._state)),
                                      "bn_newton_step")
            step()  # warm-up (captures the step's graph)
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(stream)
            for _ in range(reps):
                step()
            end.record(stream)
            end.synchronize()
            ms = start.elapsed_time(end) / reps
            times[L] = ms
            for t, s in zip(self._state_tensors(), saved):
                t.copy_(s)
            if ms < best[0]:
                if best[1] is not None:
                    self._lib.bn_model_destroy(best[1])
                best = (ms, h, L)
            else:
                self._lib.bn_model_destroy(h)
        if best[1] is not None:
            self._lib.bn_model_destroy(self._handle)
            self._handle = best[1]
            self.steps_per_thread = best[2]
        self._result = None
        return times


class MarkovSeriesBatchNewton(MarkovSeriesBatch):
    """Newton / Laplace sites for every series."""

    def __init__(self, series, **kw):
        super().__init__(series, method="newton", **kw)


def shard_series(lengths, world):
    """Partition series across `world` ranks (one GPU each) with no communication
    on the data path: longest first, each to the rank with the fewest points so
    far (greedy balancing of the scan work).  Returns one list of series indices
    per rank, each in increasing order."""
    lengths = np.asarray(lengths, dtype=np.int64)
    load = np.zeros(world, dtype=np.int64)
    parts = [[] for _ in range(world)]
    for i in np.argsort(-lengths, kind="stable"):
        r = int(np.argmin(load))
        parts[r].append(int(i))
        load[r] += lengths[i]
    return [sorted(p) for p in parts]


def gather_series_energy(local_energy, parts, rank, exchange):
    """Every rank's per-series energies back in the original series order: one
    all-gather of the ranks' vectors (`exchange.gather`, e.g. segments.TorchExchange),
    the only collective of a sharded batch, taken when the caller reads the energies."""
    local = np.zeros(max(len(p) for p in parts))
    local[:len(parts[rank])] = np.asarray(local_energy, dtype=np.float64)
    every = exchange.gather(local)
    out = np.empty(sum(len(p) for p in parts))
    for r, p in enumerate(parts):
        out[p] = np.asarray(every[r])[:len(p)]
    return out
