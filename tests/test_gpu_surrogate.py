"""Learned site expectations: the network's forward pass and loss gradient
against the float64 oracle (oracle/mlp.py), training on cubature-generated pairs,
and model steps with the learned sites against the plain cubature method."""
import numpy as np
import pytest

from tests._cases import rel_err, series

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _sur():
    import bayesnewton_gb300 as bnx
    return bnx.surrogate.CubatureSurrogate(bnx.likelihoods.HeteroscedasticNoise("exp"))


def test_mlp_forward_and_gradient_match_oracle():
    from oracle import mlp
    s = _sur()
    rng = np.random.default_rng(1)
    p = rng.normal(0, 0.2, s.num_params).astype(np.float32)
    s.set_params(p)
    n = 3000  # several split-K chunks and a ragged last one
    x = rng.normal(size=(n, 6)).astype(np.float32)
    t = rng.normal(size=(n, 6)).astype(np.float32)
    xd = torch.as_tensor(x, device="cuda")
    td = torch.as_tensor(t, device="cuda")
    out = s.forward(xd).cpu().numpy()
    o_ref, _ = mlp.forward(p.astype(np.float64), x.astype(np.float64))
    assert rel_err(out, o_ref) < 1e-5
    loss, g = s.loss_grad(xd, td)
    l_ref, g_ref = mlp.loss_grad(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - l_ref) <= 1e-5 * l_ref
    assert rel_err(g, g_ref) < 1e-4


def _hetero_model(N=4000, seed=5):
    import bayesnewton_gb300 as bnx
    K = bnx.kernels
    x, y = series(N, "hetero_exp", seed=seed)
    kern = K.Independent([K.Matern52(1.0, 2.0), K.Matern52(0.5, 5.0)])
    return bnx.models.MarkovVariationalGP(kern, bnx.likelihoods.HeteroscedasticNoise("exp"), x, y)


def test_trained_network_matches_cubature():
    m = _hetero_model()
    m.inference(lr=0.5)
    s = _sur()
    loss = s.fit(m.site_inputs(augment=4), steps=3000, batch=4096, lr=2e-3)
    assert loss < 1e-3
    raw = m.site_inputs()
    _, _, c = s.prepare(raw, ncub=32)
    pr = s.predict(raw)
    # derivatives at the model's own sites: normwise 6e-2 (the worst site), root-mean-square 2e-2
    for q in range(1, 6):
        d = (pr[:, q] - c[:, q]).cpu().double()
        ref = c[:, q].cpu().double()
        assert rel_err(pr[:, q].cpu(), ref) < 6e-2, q
        assert float(d.pow(2).mean().sqrt() / ref.pow(2).mean().sqrt()) < 2e-2, q


def test_learned_steps_against_plain_cubature():
    """After one plain step, a network trained on that posterior's sites drives
    three more VI steps; posterior and energy stay close to the plain method's
    (the surrogate error, not float32 rounding, sets the tolerance), and the
    learned site pass replaces the 400-point cubature in the step."""
    plain = _hetero_model()
    learn = _hetero_model()
    plain.inference(lr=0.5)
    learn.inference(lr=0.5)
    s = _sur()
    s.fit(learn.site_inputs(augment=4), steps=3000, batch=4096, lr=2e-3)
    learn.set_surrogate(s, spot=16, tol=0.05)
    for _ in range(3):
        plain.inference(lr=0.5)
        learn.inference(lr=0.5)
    psd, spot = learn.surrogate_counts()
    assert psd + spot < learn.num_data // 10
    assert rel_err(learn.posterior_mean.cpu(), plain.posterior_mean.cpu()) < 2e-2
    assert rel_err(learn.posterior_variance.cpu(), plain.posterior_variance.cpu()) < 2e-2
    assert abs(learn.energy() - plain.energy()) <= 2e-3 * abs(plain.energy())


def test_tensor_core_site_pass_matches_cuda_cores():
    """The learned site pass on the tensor cores (tcgen05, TF32 operands, float32
    accumulation) against the same network on CUDA cores (float32), on the sites
    of a model after one step; and the learned pass against the cubature."""
    import ctypes
    m = _hetero_model(N=20000, seed=8)
    m.inference(lr=0.5)
    s = _sur()
    s.fit(m.site_inputs(augment=2), steps=600, batch=4096, lr=2e-3)
    lib = s._lib
    n = m.num_data
    pm, pv, y = m._pm.contiguous(), m._pv.contiguous(), m.Y[:, 0].contiguous()
    out = {}
    for tc in (0, 1):
        ext = torch.empty(n, 6, device="cuda")
        cnt = (ctypes.c_uint32 * 2)()
        rc = lib.bn_mlp_sites(s._h, s._stream(), n, ctypes.c_void_p(pm.data_ptr()), ctypes.c_void_p(pv.data_ptr()),
                              ctypes.c_void_p(y.data_ptr()), 20, 0, 0.05, tc, ctypes.c_void_p(ext.data_ptr()), cnt)
        assert rc == 0
        out[tc] = (ext.cpu(), tuple(cnt))
    for q in range(6):
        assert rel_err(out[1][0][:, q], out[0][0][:, q]) < 2e-2, q
    # cubature reference at the same sites
    raw = m.site_inputs()
    _, _, c = s.prepare(raw, ncub=20)
    assert float((out[1][0][:, 1] - c[:, 1].cpu()).pow(2).mean().sqrt() / c[:, 1].cpu().pow(2).mean().sqrt()) < 5e-2


def test_learned_site_pass_is_faster_than_cubature():
    """The measured gain of the learned sites: at N = 2e5 the site pass with the
    network (tcgen05, plus the cubature fallback for the sites it hands back) takes
    less device time than the plain 20 x 20 Gauss-Hermite site pass it replaces
    (per-kernel CUDA events of the step; 0.077 against 0.097 ms measured).  The
    filter and smoother, the larger part of this configuration's step, are the same
    kernels either way."""
    plain = _hetero_model(N=200_000, seed=11)
    learn = _hetero_model(N=200_000, seed=11)
    plain.inference(lr=0.5)
    learn.inference(lr=0.5)
    s = _sur()
    s.fit(learn.site_inputs(augment=2), steps=1500, batch=4096, lr=2e-3)
    learn.set_surrogate(s, spot=64, tol=0.05)
    times = {}
    for name, m in (("plain", plain), ("learned", learn)):
        for _ in range(3):
            m.inference(lr=0.5)
        m.set_profiling(True)
        acc = []
        for _ in range(10):
            m.inference(lr=0.5)
            acc.append(m.kernel_times()["site_tail"])
        m.set_profiling(False)
        times[name] = float(np.median(acc))
    psd, spot = learn.surrogate_counts()
    assert psd + spot < learn.num_data // 5
    assert times["learned"] < 0.9 * times["plain"], times
