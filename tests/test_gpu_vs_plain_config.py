"""GPU parity on the plain regression workload at its full size (Matern52,
Gaussian noise 0.1, N = 10,000, one lr = 1 VI step, float64), through the C ABI,
against the float64 oracle (itself equal there to the exact GP:
tests/test_oracle_invariants.py), with the sequential filter / smoother (the
reference's CPU form) and with the parallel scan.

Tolerances: 1e-8 relative (normwise) on the posterior means and variances and
1e-8 relative on the energy."""
import pytest

from tests._cases import rel_err
from tests._plain_config import plain_data, plain_oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("parallel", [False, True])
def test_plain_config_full_size(parallel):
    import bayesnewton_gb300 as bnx
    x, y = plain_data()
    om, ov, oe = plain_oracle()
    gm = bnx.models.MarkovVariationalGP(bnx.kernels.Matern52(1.0, 1.0), bnx.likelihoods.Gaussian(0.1), x, y,
                                        parallel=parallel, dtype=torch.float64)
    gm.inference(lr=1.0)
    assert rel_err(gm.posterior_mean.cpu(), om) < 1e-8
    assert rel_err(gm.posterior_variance.cpu(), ov) < 1e-8
    e = gm.energy()
    assert abs(e - oe) <= 1e-8 * abs(oe), (e, oe)
