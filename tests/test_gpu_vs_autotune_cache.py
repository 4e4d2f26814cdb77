"""The batch autotuner's cache file on the GPU: a first batch times the
candidate chunk lengths and stores its choice; a second batch of the same shape
reads the choice back without timing, runs with the same chunk length, and its
step gives the same posterior (1e-6 normwise: same kernels and chunking, only
the order of float64 atomic sums may differ) and energy (1e-9 relative) as the
first."""
import numpy as np
import pytest

from tests._cases import rel_err
from tests.test_gpu_batch import _batch, make_series

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_cached_choice_matches_timed_choice(tmp_path):
    path = str(tmp_path / "tune.json")
    ss = make_series(24, 50, 3000, seed=6)
    b1 = _batch(ss, torch.float32)
    t1 = b1.autotune(cache=path)
    assert b1.steps_per_thread in t1
    b2 = _batch(ss, torch.float32)
    t2 = b2.autotune(cache=path)
    assert b2.steps_per_thread == b1.steps_per_thread
    assert t2 == {int(k): float(v) for k, v in t1.items()}
    for b in (b1, b2):
        b.inference(lr=1.0)
    assert rel_err(b2._pm.cpu(), b1._pm.cpu()) < 1e-6 and rel_err(b2._pv.cpu(), b1._pv.cpu()) < 1e-6
    e1, e2 = b1.energy(), b2.energy()
    assert abs(e1 - e2) <= 1e-9 * max(1.0, abs(e1))
    assert np.all(np.isfinite(b2.series_energy()))
