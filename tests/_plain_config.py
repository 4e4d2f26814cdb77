"""The plain regression workload at its full size: Matern52 (variance 1,
lengthscale 1, state dim 3), Gaussian noise variance 0.1, N = 10,000 sorted
inputs x ~ U[0, 100], y = sin x + 0.3 cos 3x + N(0, 0.1), one lr = 1 VI step and
the energy, float64 (the reference's CPU-runnable configuration)."""
import functools

import numpy as np

N_PLAIN = 10_000


def plain_data(seed=0):
    rng = np.random.default_rng(seed)
    x = np.sort(rng.uniform(0.0, 100.0, N_PLAIN))
    y = np.sin(x) + 0.3 * np.cos(3.0 * x) + np.sqrt(0.1) * rng.standard_normal(N_PLAIN)
    return x, y


@functools.lru_cache(maxsize=None)
def plain_oracle(seed=0):
    """Posterior mean, variance and energy of the float64 oracle after one step."""
    from oracle import kernels as OK
    from oracle import likelihoods as OL
    from oracle import models as OM
    x, y = plain_data(seed)
    m = OM.MarkovGP(OK.Matern52(1.0, 1.0), OL.Gaussian(0.1), x, y)
    m.inference(lr=1.0)
    return m.posterior_mean, m.posterior_variance, float(m.energy())
