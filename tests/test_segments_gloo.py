"""Time segments on CPU ranks (gloo, world size 2 and 3): each rank builds its
segment's filter and smoother element totals with the float64 oracle, the
totals are all-gathered over torch.distributed, and the library's host folds
(bn_segment_filter_state / bn_segment_smoother_state, no GPU) turn them into
the state entering / leaving the rank's segment; these must equal the oracle's
sequential filter and smoother states at the segment boundaries."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _flat_f(e):
    A, b, C, J, eta = e
    return np.concatenate([A.ravel(), b.ravel(), C.ravel(), J.ravel(), eta.ravel()])


def _flat_s(e):
    E, g, L = e
    return np.concatenate([E.ravel(), g.ravel(), L.ravel()])


def _case(N=257, seed=3):
    from oracle import kernels as OK
    rng = np.random.default_rng(seed)
    x = np.sort(rng.uniform(0, 60, N))
    kern = OK.Sum([OK.Matern52(1.0, 2.0), OK.Matern32(0.5, 5.0)])
    y = rng.standard_normal(N)[:, None, None]
    R = np.tile(np.array([[[0.3]]]), [N, 1, 1])
    dt = np.concatenate([[0.0], np.diff(x)])
    return kern, dt, y, R


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    from oracle import ops
    from bayesnewton_gb300 import segments
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        kern, dt, y, R = _case()
        N = dt.shape[0]
        b = segments.split_bounds(N, world)
        s, e = b[rank], b[rank + 1]
        As, Qs, H, Pinf = ops.discretise(dt, kern)
        d = Pinf.shape[0]
        # the rank's filter elements (element 0 of the series carries the prior)
        if rank == 0:
            el = ops.make_associative_filtering_elements(As[s:e], Qs[s:e], H, y[s:e], R[s:e],
                                                         np.zeros([d, 1]), Pinf)
        else:
            el = ops.parallel_filtering_element(As[s:e], Qs[s:e], H, R[s:e], y[s:e])
        tot = [x[0] for x in el]
        for i in range(1, e - s):
            tot = ops.parallel_filtering_operator_stable(tot, [x[i] for x in el])
        ex = segments.TorchExchange()
        totals = ex.gather(_flat_f(tot))
        left = segments.fold_filter(totals[:rank], d)
        # oracle filter over the whole series
        _, (fm, fP) = ops.kalman_filter(dt, kern, y, R, parallel=False)
        err_f = 0.0
        if rank > 0:
            ref = np.concatenate([fm[s - 1].ravel(), fP[s - 1].ravel()])
            err_f = float(np.max(np.abs(left - ref)) / np.max(np.abs(ref)))
        # smoother elements of the rank's steps (step k uses the transition to k+1)
        dts = np.concatenate([dt[1:], [0.0]])
        As2, Qs2, _, _ = ops.discretise(dts, kern)
        E, g, L = ops.parallel_smoothing_element(As2[s:e], Qs2[s:e], fm[s:e], fP[s:e])
        if e == N:
            E = E.copy(); g = g.copy(); L = L.copy()
            E[-1] = 0.0
            g[-1] = fm[-1]
            L[-1] = fP[-1]
        st = (E[-1], g[-1], L[-1])
        for i in range(e - s - 2, -1, -1):
            st = ops.parallel_smoothing_operator(st, (E[i], g[i], L[i]))
        stotals = ex.gather(_flat_s(st))
        right = segments.fold_smoother(stotals[rank + 1:], d)
        dtsm = np.concatenate([dt[1:], [0.0]])
        sm, sP, _ = ops.rauch_tung_striebel_smoother(dtsm, kern, fm, fP, return_full=True, parallel=False)
        err_s = 0.0
        if e < N:
            ref = np.concatenate([sm[e].ravel(), sP[e].ravel()])
            err_s = float(np.max(np.abs(right - ref)) / np.max(np.abs(ref)))
        # the smoothed state at the rank's own first step from its total and `right`
        mine = segments.fold_smoother(stotals[rank:], d)
        ref0 = np.concatenate([sm[s].ravel(), sP[s].ravel()])
        err_0 = float(np.max(np.abs(mine - ref0)) / np.max(np.abs(ref0)))
        out[rank] = (err_f, err_s, err_0)
    finally:
        dist.destroy_process_group()


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    res = {}
    _rank_main(rank, world, port, res)
    q.put((rank, res[rank]))


@pytest.mark.parametrize("world", [2, 3])
def test_segment_exchange_matches_sequential_filter_and_smoother(world):
    from bayesnewton_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from bayesnewton_gb300 import build
        build.build()
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    import queue
    import time
    results = {}
    t0 = time.time()
    while len(results) < world and time.time() - t0 < 300:
        try:
            r, v = q.get(timeout=2)
            results[r] = v
        except queue.Empty:
            if any(p.exitcode not in (None, 0) for p in procs):
                break
    for p in procs:
        p.join(timeout=60)
        if p.is_alive():
            p.terminate()
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    assert len(results) == world
    for r, (ef, es, e0) in results.items():
        assert ef < 1e-9 and es < 1e-9 and e0 < 1e-9, (r, ef, es, e0)
