#!/usr/bin/env python
"""Benchmark of the Markov-GP Newton step (sites + Kalman filter + RTS smoother +
energy) on one long series.

Workload (default): MarkovVariationalGP, Sum(Matern52, Matern32) prior (state
dim 5, variances 1.0, lengthscales 1.0), Bernoulli-logit likelihood with 20-point
Gauss-Hermite site updates, N = 1,000,000 sorted inputs x ~ U[0, 1e4],
y ~ Bernoulli(sigmoid(2 sin(x / 5))) (seeded synthetic data), parallel
(associative-scan) filter and smoother, float32 bulk arithmetic with float64
accumulation of the log marginal and energy.

One step = model.inference(lr=1): the damped natural-gradient site update from
the expectations at the current posterior, the filter (with its log marginal),
the smoother, and the site expectations / energy terms at the new posterior.
Timed on the device with CUDA events per step; L2 is flushed (a 256 MiB write)
between timed steps, outside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference's sequential float64
path (oracle/cpu_ref.cpp: lax.scan-style filter / smoother on one thread, site
expectations on all host threads) on the same workload.
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Newton step ms (sites+KF+RTS+energy) at N=1e6, learned/batched vs plain GPU"
UNIT = "ms"
N_DEFAULT = 1_000_000
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def workload(N, seed=1):
    rng = np.random.default_rng(seed)
    x = np.sort(rng.uniform(0.0, 1e4, N))
    y = (rng.uniform(size=N) < 1.0 / (1.0 + np.exp(-2.0 * np.sin(x / 5.0)))).astype(np.float64)
    return x, y


def config(N, flush=True):
    return {"workload": "MarkovVariationalGP Bernoulli-logit, Sum(Matern52,Matern32) state dim 5, N=%d, "
                        "20-pt Gauss-Hermite, parallel scan" % N,
            "num_data": N, "state_dim": 5, "site_dim": 1, "gauss_hermite_points": 20,
            "prior": "Sum(Matern52(var=1, ell=1), Matern32(var=1, ell=1))", "likelihood": "Bernoulli(logit)",
            "inference": "VI natural-gradient step, lr=1", "parallel": True,
            "l2": "flushed between timed steps (256 MiB write)" if flush else "not flushed",
            "parallelism": "replicas"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([s.strip() for s in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx.append(float(s[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return world, rank, local


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# Per-time-point algorithmic bytes of each kernel (float32 words x 4), following
# the step formula below: the filtered state handed from the filter to the smoother
# counts as d + d(d+1)/2 words each way (the library stores the 45-word smoother
# element instead, by design; ncu's traffic shows it), site = 2 words, posterior
# marginal = 2, cached derivatives g/h/lin = 3.
def kernel_bytes(d):
    rec = d + d * (d + 1) // 2
    return {
        "filter_reduce": 4 * (1 + 2 + 2 + 3),        # dt, site in, site out, g/h/lin
        "filter_rerun": 4 * (1 + 2 + 1 + rec),       # dt, site, y (mask), filtered state out
        "smoother_rerun": 4 * (rec + 2),              # filtered state in, posterior out
        "site_tail": 4 * (2 + 1 + 2 + 3),             # posterior, y, site in; g/h/lin out
    }


def step_bytes(d, p=1):
    """Algorithmic bytes of one whole step per time point (float32):
    4 [1 (dt) + p (y) + 2 s (site in/out) + s (posterior out) + 2 (d + d(d+1)/2)]."""
    s = p + p * (p + 1) // 2
    return 4 * (1 + p + 2 * s + s + 2 * (d + d * (d + 1) // 2))


def run_ours(args):
    import torch
    import bayesnewton_gb300 as bnx
    world, rank, local = dist_setup()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    N = args.num_data
    x, y = workload(N)
    kern = bnx.kernels.Sum([bnx.kernels.Matern52(1.0, 1.0), bnx.kernels.Matern32(1.0, 1.0)])
    model = bnx.models.MarkovVariationalGP(kern, bnx.likelihoods.Bernoulli("logit"), x, y,
                                           dtype=torch.float32, device=dev)
    model.update_posterior()
    for _ in range(args.warmup):
        model.inference(lr=1.0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    barrier(world)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()
            starts[i].record()
            model.inference(lr=1.0)
            ends[i].record()
        torch.cuda.synchronize()
    barrier(world)
    per = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = max_over_ranks(float(np.mean(per)), world)
    energy = model.energy()

    # dominant kernel: per-kernel CUDA events over a second timed loop
    model.set_profiling(True)
    acc = {}
    for i in range(args.steps):
        flush.zero_()
        model.inference(lr=1.0)
        for k, v in model.kernel_times().items():
            acc[k] = acc.get(k, 0.0) + v
    model.set_profiling(False)
    kavg = {k: v / args.steps for k, v in acc.items() if v > 0}
    dom = max(kavg, key=kavg.get)
    peak, peak_kind = peaks()
    d = 5
    kb = kernel_bytes(d).get(dom, 0) * N or None
    achieved = (kb / (kavg[dom] * 1e-3) / 1e9) if kb else None
    traffic = None
    prof = os.path.join(ROOT, "profiles", "kernel_traffic.json")
    if os.path.exists(prof):
        with open(prof) as f:
            traffic = json.load(f).get(dom, {}).get("dram_bytes_per_launch")

    # end to end through the public API with host buffers: H2D of the step's
    # inputs (dt, y) from pinned memory, the step, D2H of the result (energy)
    h_dt = model.dt.cpu().pin_memory()
    h_y = model.Y.cpu().pin_memory()
    h2d = h_dt.numel() * h_dt.element_size() + h_y.numel() * h_y.element_size()
    e2e = []
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        model.dt.copy_(h_dt, non_blocking=True)
        model.Y.copy_(h_y, non_blocking=True)
        model.inference(lr=1.0)
        _ = model.energy()
        e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = max_over_ranks(float(np.mean(e2e)), world)

    # prediction at N test times (seeded, uniform over the data's range): filter +
    # smoother with gains from the current sites, then the conditional per test time
    xt = torch.as_tensor(np.random.default_rng(5).uniform(x.min(), x.max(), N), device=dev)
    for _ in range(2):
        model.predict(xt)
    pe = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
    for a, b in pe:
        flush.zero_()
        a.record()
        model.predict(xt)
        b.record()
    torch.cuda.synchronize()
    pred_ms = float(np.mean([a.elapsed_time(b) for a, b in pe]))
    # hyperparameter gradient of the energy (filter + smoother with gains + the
    # per-step Fisher-identity kernel, read back to the host), wall clock
    for _ in range(2):
        model.energy_and_grad()
    gt = []
    for _ in range(3):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        model.energy_and_grad()
        gt.append((time.perf_counter() - t0) * 1e3)
    grad_ms = float(np.mean(gt))
    # the infinite-horizon model on N equidistant times (same prior, likelihood and
    # labels): one inference = two steady-state filter + smoother passes and a site
    # update (the reference's call sequence), CUDA events
    xe = np.linspace(0.0, float(x.max()), N)
    ihm = bnx.infinite_horizon.InfiniteHorizonVariationalGP(kern, bnx.likelihoods.Bernoulli("logit"), xe, y,
                                                            dtype=torch.float32, device=dev)
    for _ in range(3):
        ihm.inference(lr=1.0)
    ie = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
    for a, b in ie:
        flush.zero_()
        a.record()
        ihm.inference(lr=1.0)
        b.record()
    torch.cuda.synchronize()
    ih_ms = float(np.mean([a.elapsed_time(b) for a, b in ie]))
    del ihm

    line = {
        "metric": METRIC, "value": round(ms, 5), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 accumulation)", "data": "synthetic (seeded)",
        "config": config(N),
        "predict": {"test_times": N, "ms": round(pred_ms, 4),
                    "note": "model.predict: filter + smoother with gains + float64 conditional per test time"},
        "infinite_horizon": {"ms_per_inference": round(ih_ms, 4), "num_data": N,
                             "note": "InfiniteHorizonVariationalGP.inference on equidistant times: "
                                     "2 x (Riccati + filter + smoother + site tail) + site update"},
        "energy_grad": {"ms": round(grad_ms, 4), "params": 4,
                        "note": "model.energy_and_grad: d energy / d (variance, lengthscale) of both components, "
                                "wall clock including the host read-back"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1) if achieved else None,
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None,
                     "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": kb, "avg_launch_ms": round(kavg[dom], 5)},
        "step_roofline": {"algorithmic_bytes": step_bytes(d) * N,
                          "achieved_gbs": round(step_bytes(d) * N / (ms * 1e-3) / 1e9, 1),
                          "frac_of_hbm": round(step_bytes(d) * N / (ms * 1e-3) / 1e9 / peak, 4)},
        "kernel_ms": {k: round(v, 5) for k, v in kavg.items()},
        "e2e": {"value": round(e2e_ms, 5), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": 8 * 8 + 4},
        "gpu_launches": len(kavg) * args.steps,
        "clocks": clk.summary(),
        "energy": energy,
    }
    if rank == 0 and world == 1 and args.cpu_baseline:
        line["cpu_baseline"], port = cpu_baseline(N, samples=args.cpu_steps, return_model=True)
        del model
        line["error_vs_float64"] = error_vs_port(
            port, lambda: bnx.models.MarkovVariationalGP(kern, bnx.likelihoods.Bernoulli("logit"), x, y,
                                                         dtype=torch.float32, device=dev), args.cpu_steps)
        del port
    if world == 1 and args.sub:
        line.update(sub_workloads(args, local))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def sub_workloads(args, local):
    """The metric's other forms, measured in the same run with fewer steps:
    "plain" (the plain regression workload, float64, sequential), "batched" (4,096
    uneven series in one pass against one model per series), "learned" (the
    two-latent heteroscedastic step with learned site expectations against plain
    cubature) and "spatiotemporal" (Nt = 2000, M = 100).  Each is its own bench
    line (value, e2e, roofline, cpu_baseline); a failure is recorded, not raised."""
    import copy
    import gc
    import torch
    out = {}
    jobs = [("plain", measure_plain, {"steps": 20, "warmup": 3}),
            ("batched", measure_series, {"steps": 5, "warmup": 3, "per_series_stride": 8}),
            ("learned", measure_hetero, {"steps": 10, "warmup": 3, "fit_steps": 1500}),
            ("spatiotemporal", measure_st, {"steps": 3, "warmup": 3})]
    for name, fn, over in jobs:
        a = copy.copy(args)
        for k, v in over.items():
            setattr(a, k, v)
        t0 = time.perf_counter()
        try:
            out[name] = fn(a, 1, 0, local)
        except Exception as exc:  # the headline line is printed whatever happens here
            out[name] = {"unavailable": "%s: %s" % (type(exc).__name__, exc)}
        out[name]["wall_s"] = round(time.perf_counter() - t0, 1)
        gc.collect()
        torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------- plain regression
PLAIN_METRIC = "plain VI step ms (Matern52, Gaussian 0.1, N=10000, float64)"


def plain_workload(N=10_000, seed=0):
    """x ~ U[0, 100] sorted, y = sin x + 0.3 cos 3x + N(0, 0.1)."""
    rng = np.random.default_rng(seed)
    x = np.sort(rng.uniform(0.0, 100.0, N))
    y = np.sin(x) + 0.3 * np.cos(3.0 * x) + np.sqrt(0.1) * rng.standard_normal(N)
    return x, y


def measure_plain(args, world=1, rank=0, local=0):
    """MarkovVariationalGP, Matern52 (variance 1, lengthscale 1), Gaussian noise
    0.1, N = 10,000, one lr = 1 VI step (site update, filter with its log
    marginal, smoother, energy terms) in float64 per timed step, by the parallel
    scan; the sequential form of the same step is timed beside it."""
    import torch
    import bayesnewton_gb300 as bnx
    dev = torch.device("cuda", local)
    x, y = plain_workload()
    N = x.shape[0]

    def model(parallel):
        return bnx.models.MarkovVariationalGP(bnx.kernels.Matern52(1.0, 1.0), bnx.likelihoods.Gaussian(0.1), x, y,
                                              parallel=parallel, dtype=torch.float64, device=dev)

    def timed(m):
        for _ in range(args.warmup):
            m.inference(lr=1.0)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        torch.cuda.synchronize()
        for a0, a1 in ev:
            a0.record()
            m.inference(lr=1.0)
            a1.record()
        torch.cuda.synchronize()
        return float(np.mean([a0.elapsed_time(a1) for a0, a1 in ev]))

    # the GPU form of the step: the chunked parallel scan (float64); the sequential
    # form (one thread walks all N steps, the reference's lax.scan) is timed beside it
    m = model(True)
    with ClockSampler(local) as clk:
        ms = timed(m)
    ms_seq = timed(model(False))
    h_dt = m.dt.cpu().pin_memory()
    h_y = m.Y.cpu().pin_memory()
    e2e = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m.dt.copy_(h_dt, non_blocking=True)
        m.Y.copy_(h_y, non_blocking=True)
        m.inference(lr=1.0)
        _ = m.energy()
        e2e.append((time.perf_counter() - t0) * 1e3)
    peak, peak_kind = peaks()
    b = step_bytes(3) * N
    line = {"metric": PLAIN_METRIC, "value": round(ms, 5), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "MarkovVariationalGP, Matern52(1, 1) state dim 3, Gaussian noise 0.1, N=%d, "
                                   "x~U[0,100], y=sin x+0.3 cos 3x+N(0,0.1), VI lr=1; GPU: chunked parallel "
                                   "filter/smoother (the reference runs it sequentially)" % N,
                       "num_data": N, "state_dim": 3, "parallel": True,
                       "l2": "not flushed (1 MB of inputs and state)", "parallelism": "replicas"},
            "sequential_form_ms": round(ms_seq, 5),
            "roofline": {"bound": "latency (six dependent launches on 1 MB)",
                         "achieved": round(b / (ms * 1e-3) / 1e9, 2),
                         "peak": peak, "unit": "GB/s", "frac": round(b / (ms * 1e-3) / 1e9 / peak, 6),
                         "peak_source": peak_kind, "traffic": None, "algorithmic_bytes_per_launch": b,
                         "note": "10,000 steps are 1 MB of traffic: the step is launch- and scan-depth-bound; "
                                 "sequential_form_ms is one GPU thread walking the series in float64, which "
                                 "runs at 1/64 of the float32 rate on this GPU"},
            "e2e": {"value": round(float(np.mean(e2e)), 5), "unit": UNIT, "h2d_bytes_per_step": int(2 * 8 * N),
                    "d2h_bytes_per_step": 8 * 8 + 4},
            "clocks": clk.summary(), "energy": m.energy()}
    if rank == 0 and world == 1 and args.cpu_baseline:
        from oracle.cpu_ref import CpuRefModel
        port = CpuRefModel([("matern52", 1.0, 1.0)], 0, "gaussian", x, y, lik_variance=0.1, threads=1)
        t = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            port.step(newton=True, lr=1.0)
            t.append((time.perf_counter() - t0) * 1e3)
        line["cpu_baseline"] = {"value": round(float(np.mean(t)), 4), "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "%d full steps at N=%d (float64 C++ restatement, one thread)"
                                          % (args.steps, N), "host": host_cpu()}
        line["error_vs_float64"] = error_vs_port(port, lambda: model(True), args.steps)
    return line


def host_cpu():
    """The host CPU the baseline ran on: model (or the Arm implementer / part ids)
    and the number of logical CPUs."""
    info = {"logical_cpus": os.cpu_count(), "machine": platform.machine()}
    try:
        with open("/proc/cpuinfo") as f:
            txt = f.read()
        for key in ("model name", "CPU implementer", "CPU part"):
            for line in txt.splitlines():
                if line.lower().startswith(key.lower()):
                    info[key.replace(" ", "_").lower()] = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    return info


def cpu_baseline(N, samples=3, threads=0, return_model=False):
    from oracle.cpu_ref import CpuRefModel, load
    lib = load()
    x, y = workload(N)
    m = CpuRefModel([("matern52", 1.0, 1.0), ("matern32", 1.0, 1.0)], 0, "logit", x, y, threads=threads)
    t = []
    for _ in range(samples):
        t0 = time.perf_counter()
        m.step(newton=True, lr=1.0)
        t.append((time.perf_counter() - t0) * 1e3)
    cores = threads if threads > 0 else lib.cpuref_max_threads()
    out = {"value": round(float(np.mean(t)), 3), "unit": UNIT, "cores": cores, "kind": "port",
           "sample": "%d full steps at N=%d (float64; filter/smoother on 1 thread, sites on %d threads)"
                     % (samples, N, cores), "host": host_cpu()}
    return (out, m) if return_model else out


def error_vs_port(port, make_model, steps, lr=1.0):
    """Error of the float32 GPU step against the float64 port (oracle/cpu_ref.cpp)
    on the same inputs: a fresh model takes the same `steps` VI steps at `lr` from
    the reference's initial sites as the port did; normwise relative errors
    (max |diff| / max |port|) of the posterior means and (co)variances, the
    elementwise relative error of the means (each entry against its own size,
    entries below 1e-3 of the largest against that floor), relative error of the
    energy.  Reported, never raised: a failure is recorded."""
    try:
        g = make_model()
        for _ in range(steps):
            g.inference(lr=lr)
        pm = g.posterior_mean.double().cpu().numpy().reshape(port.pm.shape)
        pv = g.posterior_variance.double().cpu().numpy().reshape(port.pv.shape)
        e = g.energy()
        rel = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))  # noqa: E731
        floor = 1e-3
        elem = lambda a, b: float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor * np.max(np.abs(b)))))  # noqa
        return {"steps": steps, "lr": lr, "posterior_mean": rel(pm, port.pm),
                "posterior_mean_elementwise": elem(pm, port.pm), "elementwise_floor": floor,
                "posterior_variance": rel(pv, port.pv),
                "energy": abs(e - port.energy) / abs(port.energy),
                "reference": "float64 C++ restatement of the reference's step (oracle/cpu_ref.cpp)"}
    except Exception as exc:  # the bench line is printed whatever happens here
        return {"unavailable": "%s: %s" % (type(exc).__name__, exc)}


# ---------------------------------------------------------------- many series
SERIES_METRIC = "batched step ms (4096 uneven series, Matern32, Gaussian/Poisson) vs per-series launches"


def series_workload(S=4096, lmin=100, lmax=50000, seed=3):
    """S series, lengths log-uniform in [lmin, lmax], inputs sorted U[0, n]
    (unit mean spacing), Matern32 (variance 1, lengthscale log-uniform in
    [0.5, 20]) with f drawn from the prior by the exact state-space recursion;
    even series Gaussian (noise 0.05), odd series Poisson counts with rate exp(f)."""
    rng = np.random.default_rng(seed)
    lens = np.exp(rng.uniform(np.log(lmin), np.log(lmax), S)).astype(np.int64)
    ell = np.exp(rng.uniform(np.log(0.5), np.log(20.0), S))
    xs = [np.sort(rng.uniform(0.0, float(n), n)) for n in lens]
    order = np.argsort(-lens, kind="stable")  # active series are a prefix of this order
    ln, lo = lens[order], ell[order]
    lam = np.sqrt(3.0) / lo
    p11, p22 = np.ones(S), 3.0 / lo ** 2
    st = np.stack([rng.standard_normal(S) * np.sqrt(p11), rng.standard_normal(S) * np.sqrt(p22)], 1)
    xcat = np.concatenate([xs[i] for i in order])
    off = np.concatenate([[0], np.cumsum(ln)[:-1]])
    fcat = np.empty_like(xcat)
    for t in range(int(ln[0])):
        k = int(np.sum(ln > t))  # the series still running at step t
        idx = off[:k] + t
        if t > 0:
            dt = xcat[idx] - xcat[idx - 1]
            l_, e = lam[:k], np.exp(-lam[:k] * dt)
            a11, a12, a21, a22 = e * (1 + l_ * dt), e * dt, -e * l_ * l_ * dt, e * (1 - l_ * dt)
            q11 = p11[:k] - (a11 * a11 * p11[:k] + a12 * a12 * p22[:k])
            q12 = -(a11 * a21 * p11[:k] + a12 * a22 * p22[:k])
            q22 = p22[:k] - (a21 * a21 * p11[:k] + a22 * a22 * p22[:k])
            l11 = np.sqrt(np.maximum(q11, 0.0))
            l21 = np.where(l11 > 1e-12, q12 / np.maximum(l11, 1e-12), 0.0)  # dt = 0: Q = 0
            l22 = np.sqrt(np.maximum(q22 - l21 * l21, 0.0))
            z1, z2 = rng.standard_normal(k), rng.standard_normal(k)
            m1 = a11 * st[:k, 0] + a12 * st[:k, 1]
            m2 = a21 * st[:k, 0] + a22 * st[:k, 1]
            st[:k, 0] = m1 + l11 * z1
            st[:k, 1] = m2 + l21 * z1 + l22 * z2
        fcat[idx] = st[:k, 0]
    f = [None] * S
    for j, i in enumerate(order):
        f[i] = fcat[off[j]:off[j] + ln[j]]
    out = []
    for i in range(S):
        if i % 2 == 0:
            y = f[i] + np.sqrt(0.05) * rng.standard_normal(lens[i])
            out.append(("gaussian", 0.05, float(ell[i]), xs[i], y))
        else:
            y = rng.poisson(np.exp(f[i])).astype(np.float64)
            out.append(("poisson", 1.0, float(ell[i]), xs[i], y))
    return out


def series_config(S, total):
    return {"workload": "%d independent series, lengths log-uniform [100, 50000] (N=%d total), Matern32 "
                        "(state dim 2, lengthscales log-uniform [0.5, 20]), half Gaussian (noise 0.05), half "
                        "Poisson(exp f), f drawn from the prior; VI step lr=1, one batched pass" % (S, total),
            "num_series": S, "num_data": total, "state_dim": 2, "site_dim": 1,
            "l2": "inputs and state larger than L2 (%.1f GB of sites, posterior and scan state)"
                  % (total * 4 * 20 / 1e9),
            "parallelism": "replicas"}


def measure_series(args, world=1, rank=0, local=0):
    import torch
    import bayesnewton_gb300 as bnx
    dev = torch.device("cuda", local)
    data = series_workload(args.num_series)
    K, L = bnx.kernels, bnx.likelihoods

    def objs(lk, nv, ell):
        return K.Matern32(1.0, ell), (L.Gaussian(nv) if lk == "gaussian" else L.Poisson())

    series = [(*objs(lk, nv, ell), x, y) for lk, nv, ell, x, y in data]
    total = int(sum(len(s[2]) for s in series))
    model = bnx.batch.MarkovSeriesBatch(series, dtype=torch.float32, device=dev)
    model.update_posterior()
    tune = model.autotune()
    for _ in range(args.warmup):
        model.inference(lr=1.0)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    barrier(world)
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            starts[i].record()
            model.inference(lr=1.0)
            ends[i].record()
        torch.cuda.synchronize()
    barrier(world)
    ms = max_over_ranks(float(np.mean([s.elapsed_time(e) for s, e in zip(starts, ends)])), world)

    model.set_profiling(True)
    acc = {}
    for i in range(args.steps):
        model.inference(lr=1.0)
        for k, v in model.kernel_times().items():
            acc[k] = acc.get(k, 0.0) + v
    model.set_profiling(False)
    kavg = {k: v / args.steps for k, v in acc.items() if v > 0}
    dom = max(kavg, key=kavg.get)
    peak, peak_kind = peaks()
    kb = kernel_bytes(2).get(dom, 0) * total or None
    achieved = (kb / (kavg[dom] * 1e-3) / 1e9) if kb else None

    # the same work as one model per series, stepped one after another (what a
    # caller of the single-series API does); each model's step is its own graph
    # (every `stride`-th series when a sample is asked for, scaled to all series:
    # the workload's series are in random length order)
    stride = max(1, int(getattr(args, "per_series_stride", 1)))
    singles = []
    for kern, lik, x, y in series[::stride]:
        g = bnx.models.MarkovVariationalGP(kern, lik, x, y, dtype=torch.float32, device=dev)
        g.update_posterior()
        singles.append(g)
    for g in singles:
        g.inference(lr=1.0)
    torch.cuda.synchronize()
    per_series = []
    for _ in range(max(1, min(args.steps, 3))):
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        for g in singles:
            g.inference(lr=1.0)
        t1.record()
        t1.synchronize()
        per_series.append(t0.elapsed_time(t1))
    ms_single = float(np.mean(per_series)) * len(series) / len(singles)
    n_single = len(singles)
    del singles

    # end to end: H2D of (dt, y), the step, D2H of the per-series energies
    h_dt = model.dt.cpu().pin_memory()
    h_y = model.Y.cpu().pin_memory()
    h2d = h_dt.numel() * h_dt.element_size() + h_y.numel() * h_y.element_size()
    e2e = []
    for i in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        model.dt.copy_(h_dt, non_blocking=True)
        model.Y.copy_(h_y, non_blocking=True)
        model.inference(lr=1.0)
        _ = model.series_energy()
        e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = max_over_ranks(float(np.mean(e2e)), world)
    line = {
        "metric": SERIES_METRIC, "value": round(ms, 5), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 accumulation)", "data": "synthetic (seeded)",
        "config": series_config(len(series), total),
        "per_series_launch_ms": round(ms_single, 3), "batched_speedup": round(ms_single / ms, 2),
        "per_series_sample": "%d of %d series stepped one model at a time%s" % (
            n_single, len(series), "" if n_single == len(series) else ", scaled by the series count"),
        "autotune_ms": {str(k): round(v, 4) for k, v in tune.items()}, "steps_per_thread": model.steps_per_thread,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1) if achieved else None,
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None,
                     "peak_source": peak_kind, "traffic": None,
                     "algorithmic_bytes_per_launch": kb, "avg_launch_ms": round(kavg[dom], 5)},
        "step_roofline": {"algorithmic_bytes": step_bytes(2) * total,
                          "achieved_gbs": round(step_bytes(2) * total / (ms * 1e-3) / 1e9, 1),
                          "frac_of_hbm": round(step_bytes(2) * total / (ms * 1e-3) / 1e9 / peak, 4)},
        "kernel_ms": {k: round(v, 5) for k, v in kavg.items()},
        "e2e": {"value": round(e2e_ms, 5), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": 8 * len(series)},
        "gpu_launches": len(kavg) * args.steps,
        "clocks": clk.summary(),
        "energy": model.energy(),
        "series_nonfinite_energy": int(np.sum(~np.isfinite(model.series_energy()))),
        "status": model.status(),
    }
    if rank == 0 and world == 1 and args.cpu_baseline:
        line["cpu_baseline"] = series_cpu_baseline(data, total)
    return line


def run_series(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(torch.device("cuda", local))
    line = measure_series(args, world, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def series_cpu_baseline(data, total, budget_s=15.0):
    """The float64 C++ port, one series at a time on one thread each, over all host
    threads (series are independent), on a bounded sample of series; scaled to the
    whole batch by time points."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle.cpu_ref import CpuRefModel, load
    load()
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    models = []
    done = 0
    for lk, nv, ell, x, y in data:
        models.append(CpuRefModel([("matern32", 1.0, ell)], 0, lk, x, y, lik_variance=nv, threads=1))
        done += len(x)
        if done >= total // 8:
            break
    t0 = time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:
        list(ex.map(lambda m: m.step(newton=True, lr=1.0), models))
    dt = time.perf_counter() - t0
    return {"value": round(dt * 1e3 * total / done, 3), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "one step of the first %d series (%d of %d time points, float64), %d threads, "
                      "scaled to all series by time points" % (len(models), done, total, cores)}


# ---------------------------------------------------------------- spatio-temporal
ST_METRIC = "spatio-temporal VI step ms (Nt=2000, M=100 inducing, 500 obs/step, state dim 200)"


def st_workload(Nt=2000, g=10, Nr=500, lt=20.0, ls=0.3, seed=5):
    """Nt unit-spaced time points, M = g x g inducing inputs on [0.05, 0.95]^2,
    Nr observations per time point at x ~ U[0,1]^2, Matern32 (time, variance 1,
    lengthscale lt) x Matern32 (space, variance 1, lengthscale ls); f drawn from
    the prior through the state-space form (u(t) by the exact temporal recursion,
    f = B u + sqrt(diag C) e, i.e. the FIC marginals); y ~ Poisson(exp f)."""
    rng = np.random.default_rng(seed)
    z1 = np.linspace(0.05, 0.95, g)
    za, zb = np.meshgrid(z1, z1)
    z = np.stack([za.ravel(), zb.ravel()], 1)
    M = z.shape[0]
    X = np.arange(Nt, dtype=np.float64)
    R = rng.uniform(0.0, 1.0, [Nt, Nr, 2])

    def k32(a, b, ell):
        r = np.sqrt(np.maximum(np.sum((a[:, None, :] - b[None, :, :]) ** 2, -1), 1e-36)) / ell
        return (1 + np.sqrt(3) * r) * np.exp(-np.sqrt(3) * r)

    L = np.linalg.cholesky(k32(z, z, ls) + 1e-10 * np.eye(M))
    lam = np.sqrt(3.0) / lt
    e = np.exp(-lam)
    A = e * np.array([[1 + lam, 1.0], [-lam * lam, 1 - lam]])
    Pinf = np.diag([1.0, lam * lam])
    Q = Pinf - A @ Pinf @ A.T
    Lq = np.linalg.cholesky(Q)
    x = np.linalg.cholesky(Pinf) @ rng.standard_normal([2, M])
    f = np.empty([Nt, Nr])
    for t in range(Nt):
        if t > 0:
            x = A @ x + Lq @ rng.standard_normal([2, M])
        Krz = k32(R[t], z, ls)
        B = np.linalg.solve(L, Krz.T).T
        c = np.maximum(1.0 - np.sum(B * B, 1), 0.0)
        f[t] = B @ x[0] + np.sqrt(c) * rng.standard_normal(Nr)
    Y = rng.poisson(np.exp(f)).astype(np.float64)
    return z, X, R, Y, lt, ls


def st_config(Nt, M, Nr):
    return {"workload": "spatio-temporal VGP, Nt=%d, M=%d inducing (10x10 grid), %d obs/step at x~U[0,1]^2, "
                        "Matern32-time x Matern32-space (state dim %d), Poisson(exp f), f from the prior; "
                        "VI step lr=1" % (Nt, M, Nr, 2 * M),
            "num_time": Nt, "num_inducing": M, "obs_per_step": Nr, "state_dim": 2 * M,
            "l2": "inputs and scan state larger than L2 (~%.1f GB of element arrays)" % (Nt * (2 * M) ** 2 * 4 * 10 / 1e9),
            "parallelism": "replicas"}


def st_flops(Nt, M, Nr, S=2):
    """Dense flops of one step as the reference computes it (2 n^3 per n x n
    product, d = S M, q = M): KF + RTS + sites per time point."""
    d, q = S * M, M
    kf = 2 * d ** 3 + 2 * q * d * d + 2 * q * q * d + q ** 3 / 3 + 2 * q * q * d + 2 * q * d * d
    rts = 4 * d ** 3 + d ** 3 / 3 + 2 * d ** 3
    sites = 2 * 2 * Nr * M * M
    return (kf + rts + sites) * Nt


def measure_st(args, world=1, rank=0, local=0):
    import torch
    import bayesnewton_gb300 as bnx
    dev = torch.device("cuda", local)
    Nt = args.num_time
    z, X, R, Y, lt, ls = st_workload(Nt=Nt)
    M, Nr = z.shape[0], Y.shape[1]
    kern = bnx.kernels.SpatioTemporalMatern32(1.0, lt, ls, z=z)
    model = bnx.models.MarkovVariationalGP(kern, bnx.likelihoods.Poisson(), X, Y, R=R)
    model.update_posterior()
    for _ in range(args.warmup):
        model.inference(lr=1.0)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    barrier(world)
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            starts[i].record()
            model.inference(lr=1.0)
            ends[i].record()
        torch.cuda.synchronize()
    barrier(world)
    ms = max_over_ranks(float(np.mean([s.elapsed_time(e) for s, e in zip(starts, ends)])), world)
    h_y = model.Y.cpu().pin_memory()
    h_dt = model.dt.cpu().pin_memory()
    e2e = []
    for i in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        model.Y.copy_(h_y, non_blocking=True)
        model.dt.copy_(h_dt, non_blocking=True)
        model.inference(lr=1.0)
        _ = model.energy()
        e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = max_over_ranks(float(np.mean(e2e)), world)
    fl = st_flops(Nt, M, Nr)
    roof = st_gemm_roofline(dev)
    line = {
        "metric": ST_METRIC, "value": round(ms, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": st_config(Nt, M, Nr),
        "dense_reference_flops": fl, "dense_equiv_tflops": round(fl / (ms * 1e-3) / 1e12, 3),
        "roofline": roof,
        "e2e": {"value": round(e2e_ms, 4), "unit": UNIT, "h2d_bytes_per_step": int(h_y.numel() * 4 + h_dt.numel() * 4),
                "d2h_bytes_per_step": 8 * 8 + 4},
        "clocks": clk.summary(), "energy": model.energy(), "status": model.status(),
    }
    if rank == 0 and world == 1 and args.cpu_baseline:
        line["cpu_baseline"] = st_cpu_baseline(args.st_cpu_time)
    return line


def st_gemm_roofline(dev):
    """Roofline of the step's dominant kernel, the tensor-core batched product,
    timed live through the C ABI (bn_dense_gemm) at the filter scan's bottom-level
    shape (1024 products of 200 x 200 x 200; 164 MB per operand, above L2): its
    TF32 MMA rate (3 MMAs per product in 3xTF32) against cuBLAS's TF32 rate on this
    GPU, measured here the same way as bench.py --workload peaks."""
    import ctypes
    import torch
    from bayesnewton_gb300 import _lib
    lib = _lib.load()
    nb, n = 1024, 200
    g = torch.Generator(device=dev).manual_seed(0)
    A = torch.randn(nb, n, n, device=dev, generator=g)
    B = torch.randn(nb, n, n, device=dev, generator=g)
    C = torch.empty(nb, n, n, device=dev)
    s = torch.cuda.current_stream(dev).cuda_stream

    def call():
        return lib.bn_dense_gemm(ctypes.c_void_p(s), 1, nb, 0, 0, n, n, n, 1.0, ctypes.c_void_p(A.data_ptr()),
                                 ctypes.c_void_p(B.data_ptr()), 0.0, None, ctypes.c_void_p(C.data_ptr()))

    for _ in range(3):
        if call() != 0:
            return None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(10):
        call()
    e1.record()
    torch.cuda.synchronize()
    gemm_ms = e0.elapsed_time(e1) / 10
    result = 2.0 * nb * n ** 3 / (gemm_ms * 1e-3) / 1e12
    del A, B, C
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    a = torch.randn(8192, 8192, device=dev)
    b = torch.randn(8192, 8192, device=dev)
    for _ in range(3):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(5):
        torch.matmul(a, b)
    e1.record()
    torch.cuda.synchronize()
    tf32 = 2.0 * 8192 ** 3 / (e0.elapsed_time(e1) / 5 * 1e-3) / 1e12
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b
    traffic = None
    prof = os.path.join(ROOT, "profiles", "kernel_traffic.json")
    if os.path.exists(prof):
        with open(prof) as f:
            traffic = json.load(f).get("tc_bgemm", {}).get("dram_bytes_per_launch")
    return {"bound": "tensor", "kernel": "tc_bgemm: 3xTF32 tcgen05 products, 1024 x 200 x 200 x 200 "
                                         "(the filter scan's bottom level; operands above L2)",
            "achieved": round(3 * result, 1), "peak": round(tf32, 1), "unit": "TFLOP/s",
            "frac": round(3 * result / tf32, 4), "peak_source": "cuBLAS TF32 8192^3 (torch.matmul), measured here",
            "result_tflops": round(result, 1), "avg_launch_ms": round(gemm_ms, 4), "traffic": traffic,
            "note": "achieved = TF32 MMA work (3 products per result product) per launch / launch time"}


def run_st(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(torch.device("cuda", local))
    line = measure_st(args, world, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def st_cpu_baseline(nt_sample):
    """The float64 oracle (numpy, sequential filter / smoother as the reference's
    CPU path) on the first nt_sample time points, scaled to Nt = 2000 by time points."""
    from oracle import kernels as OK, likelihoods as OL
    from oracle.spatiotemporal import SpatioTemporalKernel, STMarkovGP
    z, X, R, Y, lt, ls = st_workload(Nt=nt_sample)
    om = STMarkovGP(SpatioTemporalKernel(OK.Matern32(1.0, lt), OK.Matern32(1.0, ls), z), OL.Poisson(), X, R, Y)
    t0 = time.perf_counter()
    om.inference(lr=1.0)
    om.energy()
    dt = time.perf_counter() - t0
    return {"value": round(dt * 1e3 * 2000 / nt_sample, 1), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "one VI step + energy of the float64 numpy oracle on %d of 2000 time points (sequential "
                      "KF/RTS, numpy BLAS threads), scaled by time points" % nt_sample}


# ---------------------------------------------------------------- heteroscedastic
HET_METRIC = "heteroscedastic VI step ms (2 latent Matern52, N=200000, 20x20 Gauss-Hermite sites)"


def matern52_prior_draw(x, var, ell, rng):
    """f(x) from the Matern52 prior by the exact state-space recursion (sorted x)."""
    lam = np.sqrt(5.0) / ell
    kp = 5.0 / 3.0 * var / ell ** 2
    Pinf = np.array([[var, 0.0, -kp], [0.0, kp, 0.0], [-kp, 0.0, 25.0 * var / ell ** 4]])
    st = np.linalg.cholesky(Pinf) @ rng.standard_normal(3)
    f = np.empty(x.shape[0])
    f[0] = st[0]
    F = np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [-lam ** 3, -3 * lam ** 2, -3 * lam]])
    from scipy.linalg import expm
    dts = np.diff(x)
    z = rng.standard_normal([x.shape[0], 3])
    for n in range(1, x.shape[0]):
        A = expm(F * dts[n - 1])
        Q = Pinf - A @ Pinf @ A.T
        w, V = np.linalg.eigh(0.5 * (Q + Q.T))
        st = A @ st + V @ (np.sqrt(np.maximum(w, 0.0)) * z[n])
        f[n] = st[0]
    return f


def hetero_workload(N=200_000, seed=7):
    """x ~ U[0, 1000] sorted; f1 ~ Matern52(var 1, ell 10), f2 ~ Matern52(var 0.25,
    ell 20) from the prior; y = f1 + exp(f2) e."""
    rng = np.random.default_rng(seed)
    x = np.sort(rng.uniform(0.0, 1000.0, N))
    f1 = matern52_prior_draw(x, 1.0, 10.0, rng)
    f2 = matern52_prior_draw(x, 0.25, 20.0, rng)
    y = f1 + np.exp(f2) * rng.standard_normal(N)
    return x, y


def measure_hetero(args, world=1, rank=0, local=0):
    import torch
    import bayesnewton_gb300 as bnx
    dev = torch.device("cuda", local)
    x, y = hetero_workload(args.num_hetero)
    K = bnx.kernels
    kern = K.Independent([K.Matern52(1.0, 10.0), K.Matern52(0.25, 20.0)])
    model = bnx.models.MarkovVariationalGP(kern, bnx.likelihoods.HeteroscedasticNoise("exp"), x, y,
                                           dtype=torch.float32, device=dev)
    model.update_posterior()
    for _ in range(args.warmup):
        model.inference(lr=0.5)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            starts[i].record()
            model.inference(lr=0.5)
            ends[i].record()
        torch.cuda.synchronize()
    ms = float(np.mean([s.elapsed_time(e) for s, e in zip(starts, ends)]))
    model.set_profiling(True)
    acc = {}
    for i in range(args.steps):
        model.inference(lr=0.5)
        for k, v in model.kernel_times().items():
            acc[k] = acc.get(k, 0.0) + v
    model.set_profiling(False)
    kavg = {k: round(v / args.steps, 5) for k, v in acc.items() if v > 0}

    # the learned sites: a second model trained on its own posterior after one
    # plain step, then stepped with the network in place of the cubature
    learn = bnx.models.MarkovVariationalGP(kern, bnx.likelihoods.HeteroscedasticNoise("exp"), x, y,
                                           dtype=torch.float32, device=dev)
    ref = bnx.models.MarkovVariationalGP(kern, bnx.likelihoods.HeteroscedasticNoise("exp"), x, y,
                                         dtype=torch.float32, device=dev)
    learn.inference(lr=0.5)
    ref.inference(lr=0.5)
    sur = bnx.surrogate.CubatureSurrogate(bnx.likelihoods.HeteroscedasticNoise("exp"), device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fit_loss = sur.fit(learn.site_inputs(augment=2), steps=args.fit_steps, batch=4096, lr=2e-3)
    torch.cuda.synchronize()
    fit_s = time.perf_counter() - t0
    learn.set_surrogate(sur, spot=64, tol=0.05)
    for _ in range(args.warmup):
        learn.inference(lr=0.5)
        ref.inference(lr=0.5)
    ls_, le_ = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)], \
        [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for i in range(args.steps):
        ls_[i].record()
        learn.inference(lr=0.5)
        le_[i].record()
        ref.inference(lr=0.5)
    torch.cuda.synchronize()
    ms_learn = float(np.mean([a.elapsed_time(b) for a, b in zip(ls_, le_)]))
    learn.set_profiling(True)
    lacc = {}
    for i in range(args.steps):
        learn.inference(lr=0.5)
        ref.inference(lr=0.5)
        for k, v in learn.kernel_times().items():
            lacc[k] = lacc.get(k, 0.0) + v
    learn.set_profiling(False)
    psd, spot = learn.surrogate_counts()
    pm_l, pm_r = learn.posterior_mean.reshape(-1).double(), ref.posterior_mean.reshape(-1).double()
    learned = {"ms_per_step": round(ms_learn, 5), "speedup_vs_plain": round(ms / ms_learn, 3),
               "kernel_ms": {k: round(v / args.steps, 5) for k, v in lacc.items() if v > 0},
               "fit_seconds": round(fit_s, 2), "fit_loss": fit_loss,
               "fallback_sites": {"precision": psd, "spot_check": spot, "of": int(args.num_hetero)},
               "vs_plain_same_steps": {
                   "posterior_mean_rel": float((pm_l - pm_r).abs().max() / pm_r.abs().max()),
                   "energy_rel": abs(learn.energy() - ref.energy()) / abs(ref.energy())}}
    line = {"metric": HET_METRIC, "value": round(ms, 5), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "HeteroscedasticNoise(exp), Independent(Matern52(1, 10), Matern52(0.25, 20)) "
                                   "state dim 6, N=%d, x~U[0,1000], f from the prior, 20x20 Gauss-Hermite, "
                                   "VI lr=0.5 (lr=1 oscillates on this model in float64 as well)" % args.num_hetero, "num_data": args.num_hetero, "state_dim": 6,
                       "site_dim": 2, "parallelism": "replicas"},
            "kernel_ms": kavg, "clocks": clk.summary(), "energy": model.energy(), "status": model.status(),
            "learned_sites": learned}
    if rank == 0 and world == 1 and args.cpu_baseline:
        del model, learn, ref
        line["cpu_baseline"], port = hetero_cpu_baseline(x, y, args.cpu_steps)
        line["error_vs_float64"] = error_vs_port(
            port, lambda: bnx.models.MarkovVariationalGP(kern, bnx.likelihoods.HeteroscedasticNoise("exp"), x, y,
                                                         dtype=torch.float32, device=dev), args.cpu_steps, lr=0.5)
    return line


def run_hetero(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(torch.device("cuda", local))
    line = measure_hetero(args, world, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def hetero_cpu_baseline(x, y, steps):
    """The float64 C++ port of the two-latent heteroscedastic VI step (20 x 20
    Gauss-Hermite sites on every host thread, the filter / smoother on one), timed
    over `steps` lr = 0.5 steps of the full workload; returns (baseline, port)."""
    from oracle.cpu_ref import CpuRefModel, load
    load()
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    port = CpuRefModel([("matern52", 1.0, 10.0), ("matern52", 0.25, 20.0)], 1, "hetero_exp", x, y, threads=cores)
    t = []
    for _ in range(steps):
        t0 = time.perf_counter()
        port.step(newton=True, lr=0.5)
        t.append((time.perf_counter() - t0) * 1e3)
    return ({"value": round(float(np.mean(t)), 3), "unit": UNIT, "cores": cores, "kind": "port",
             "sample": "%d full steps at N=%d (float64; 20x20 Gauss-Hermite sites on %d threads, filter / smoother "
                       "on 1)" % (steps, x.shape[0], cores), "host": host_cpu()}, port)


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.cpu_ref import CpuRefModel, load
    load()
    N = args.num_data
    x, y = workload(N)
    # every host thread this process may run on (torchrun sets OMP_NUM_THREADS=1
    # for its ranks; rank 0 runs alone here, so it takes the whole host)
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    m = CpuRefModel([("matern52", 1.0, 1.0), ("matern32", 1.0, 1.0)], 0, "logit", x, y, threads=cores)
    # bounded: at most this many timed steps (each a full N-point step)
    K = min(args.steps, args.ref_max_steps)
    W = min(args.warmup, 3)
    for _ in range(W):
        m.step(newton=True, lr=1.0)
    t = []
    for _ in range(K):
        t0 = time.perf_counter()
        m.step(newton=True, lr=1.0)
        t.append((time.perf_counter() - t0) * 1e3)
    ms = float(np.mean(t))
    line = {"metric": METRIC, "value": round(ms, 3), "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded)", "config": config(N, flush=False), "impl": "reference",
            "cpu_baseline": {"value": round(ms, 3), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d full steps at N=%d (float64 C++ restatement; filter/smoother on "
                                       "1 thread as lax.scan, sites on %d threads)" % (K, N, cores),
                             "host": host_cpu()},
            "e2e": {"value": round(ms, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "energy": float(m.energy)}
    print(json.dumps(line), flush=True)


def run_peaks(args):
    """The matmul throughput of this GPU's library GEMMs for the precisions the
    kernels here use beside bf16 (which MEASURED_PEAKS.json holds): float32 on the
    CUDA cores, TF32 on the tensor cores, float64.  Square products, CUDA events,
    3 warm-up and `--steps` timed products each."""
    import torch
    dev = torch.device("cuda", 0)
    out = {}
    for name, dtype, n, tf32 in (("fp32", torch.float32, 8192, False), ("tf32", torch.float32, 8192, True),
                                 ("fp64", torch.float64, 4096, False)):
        torch.backends.cuda.matmul.allow_tf32 = tf32
        a = torch.randn(n, n, device=dev, dtype=dtype)
        b = torch.randn(n, n, device=dev, dtype=dtype)
        for _ in range(3):
            torch.matmul(a, b)
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s0.record()
        for _ in range(args.steps):
            torch.matmul(a, b)
        s1.record()
        torch.cuda.synchronize()
        ms = s0.elapsed_time(s1) / args.steps
        out[name] = {"n": n, "ms": round(ms, 4), "tflops": round(2.0 * n ** 3 / (ms * 1e-3) / 1e12, 2)}
        del a, b
    torch.backends.cuda.matmul.allow_tf32 = False
    print(json.dumps({"metric": "library GEMM throughput (torch.matmul / cuBLAS)", "unit": "TFLOP/s",
                      "peaks": out, "device": torch.cuda.get_device_name(0)}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--num-data", type=int, default=N_DEFAULT)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--ref-max-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--workload", default="long", choices=["long", "series", "st", "hetero", "peaks"],
                    help="long: one series of --num-data points; series: --num-series uneven series; "
                         "st: the spatio-temporal model")
    ap.add_argument("--num-series", type=int, default=4096)
    ap.add_argument("--num-time", type=int, default=2000)
    ap.add_argument("--num-hetero", type=int, default=200_000)
    ap.add_argument("--fit-steps", type=int, default=3000, help="hetero: training steps of the learned sites")
    ap.add_argument("--st-cpu-time", type=int, default=200)
    ap.add_argument("--no-sub", dest="sub", action="store_false",
                    help="long workload: skip the plain / batched / learned / spatio-temporal sub-lines")
    ap.add_argument("--per-series-stride", type=int, default=1,
                    help="series: step every k-th series alone for the per-series comparison")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "series":
        run_series(args)
    elif args.workload == "st":
        run_st(args)
    elif args.workload == "hetero":
        run_hetero(args)
    elif args.workload == "peaks":
        run_peaks(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
