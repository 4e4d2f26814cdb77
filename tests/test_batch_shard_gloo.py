"""Sharding many series across ranks (one GPU each, no collective on the data
path): the partition covers every series once with balanced point counts, and
the per-series energies gathered over a gloo process group of 2 or 3 CPU ranks come
back in the original order.  No GPU: each rank's energies are a deterministic
function of its series (what each rank's MarkovSeriesBatch would report)."""
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lengths(S=97, seed=0):
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(100), np.log(5e4), S)).astype(np.int64)


def test_shard_covers_and_balances():
    sys.path.insert(0, ROOT)
    from bayesnewton_gb300.batch import shard_series
    L = _lengths()
    for world in (1, 2, 3, 8):
        parts = shard_series(L, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(L)))
        loads = [int(L[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= int(L.max())


def _worker(rank, world, port, q):
    try:
        import torch.distributed as dist
        sys.path.insert(0, ROOT)
        from bayesnewton_gb300.batch import gather_series_energy, shard_series
        from bayesnewton_gb300.segments import TorchExchange
        dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
        L = _lengths()
        parts = shard_series(L, world)
        local = [float(np.sin(i) * L[i]) for i in parts[rank]]  # stands in for the rank's batch energies
        out = gather_series_energy(local, parts, rank, TorchExchange())
        q.put((rank, out))
        dist.destroy_process_group()
    except Exception as e:  # report to the parent instead of hanging it
        q.put((rank, repr(e)))


@pytest.mark.parametrize("world", [2, 3])
def test_gather_series_energy_gloo(world):
    import multiprocessing as mp
    import socket
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = {}
    import queue
    for _ in range(world):
        try:
            r, out = q.get(timeout=120)
        except queue.Empty:
            break
        got[r] = out
    for p in procs:
        p.join(timeout=30)
        if p.is_alive():
            p.kill()
    assert len(got) == world, got
    L = _lengths()
    expect = np.array([np.sin(i) * L[i] for i in range(len(L))])
    for r in range(world):
        assert not isinstance(got[r], str), got[r]
        np.testing.assert_allclose(got[r], expect, rtol=0, atol=0)
