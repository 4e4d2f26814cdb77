"""Full-size parity of the many-series step: the 4,096-series workload of
bench.py --workload series (lengths log-uniform in [100, 50,000], 32.8 M time
points, Matern32 with lengthscales log-uniform in [0.5, 20], half Gaussian noise
0.05 and half Poisson counts, f drawn from the prior), float32, two VI steps at
lr = 1 in one batched pass.

Series are independent, so the size-independent property is that each series of
the full batch equals the float64 C++ restatement of the reference's step
(oracle/cpu_ref.cpp) run on that series alone: checked on 46 series (every 97th,
the shortest and the two longest) with the tolerances of tests/test_gpu_batch.py
(2e-4 normwise relative on posterior means, 1e-5 relative on each series'
energy).  Over all 4,096 series: finite energies whose sum is the batch energy
(1e-5 relative, the two sums accumulate in different orders and precisions),
finite means and positive variances."""
import numpy as np
import pytest

from tests._cases import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_full_size_series_batch_against_port():
    import bayesnewton_gb300 as bnx
    from bench import series_workload
    from oracle.cpu_ref import CpuRefModel
    data = series_workload(4096)
    K, L = bnx.kernels, bnx.likelihoods
    series = [(K.Matern32(1.0, ell), L.Gaussian(nv) if lk == "gaussian" else L.Poisson(), x, y)
              for lk, nv, ell, x, y in data]
    b = bnx.batch.MarkovSeriesBatch(series, dtype=torch.float32)
    for _ in range(2):
        b.inference(lr=1.0)
    se = b.series_energy()
    total = b.energy()
    assert np.all(np.isfinite(se))
    assert abs(float(np.sum(se)) - total) <= 1e-5 * max(1.0, abs(total)), (float(np.sum(se)), total)
    assert torch.isfinite(b._pm).all() and bool((b._pv > 0).all())
    lens = np.array([len(s[3]) for s in data])
    order = np.argsort(lens, kind="stable")
    pick = sorted(set(range(0, len(data), 97)) | {int(order[0]), int(order[-1]), int(order[-2])})
    pm = b._pm[:, 0].cpu().numpy()
    errs = []
    for i in pick:
        lk, nv, ell, x, y = data[i]
        ref = CpuRefModel([("matern32", 1.0, ell)], 0, lk, x, y, lik_variance=nv, threads=1)
        for _ in range(2):
            ref.step(newton=True, lr=1.0)
        errs.append(rel_err(pm[b.series_slice(i)], ref.pm.reshape(-1)))
        e_ref = ref.result[0]
        assert abs(se[i] - e_ref) <= 1e-5 * max(1.0, abs(e_ref)), (i, len(x), lk, se[i], e_ref)
    assert max(errs) < 2e-4, (max(errs), pick[int(np.argmax(errs))])
