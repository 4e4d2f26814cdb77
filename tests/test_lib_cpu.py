"""Host-side checks that need no GPU: the C-ABI library loads and exports every
symbol include/bnx.h declares, and the ctypes structures match the header."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _built():
    from bayesnewton_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from bayesnewton_gb300 import build
        build.build()
    return _lib.load()


def test_library_exports_every_declared_symbol():
    lib = _built()
    decl = set(re.findall(r"\b(bn_\w+)\s*\(", open(os.path.join(ROOT, "include", "bnx.h")).read()))
    assert decl, "no declarations found"
    missing = sorted(d for d in decl if not hasattr(lib, d))
    assert not missing, missing
    assert b"sm_103a" in lib.bn_build_info()


def test_struct_layouts_match_header():
    from bayesnewton_gb300 import _lib
    # int32 x 2 + int32[8] x 2 + double[8] x 2 + double[64] x 2
    assert ctypes.sizeof(_lib.PriorDesc) == 8 + 64 + 128 + 1024
    assert ctypes.sizeof(_lib.LikDesc) == 20 + 4 + 24
    assert ctypes.sizeof(_lib.SiteState) == 7 * 8
    assert ctypes.sizeof(_lib.StDesc) == 72


def test_gauss_hermite_matches_numpy():
    """The library's Gauss-Hermite rule equals numpy's hermgauss, which the
    reference calls (bayesnewton/cubature.py:6, 70), after its sqrt(2) and
    1/sqrt(pi) scaling (cubature.py:76-84)."""
    import numpy as np
    lib = _built()
    for n in (1, 2, 5, 20, 32):
        x = (ctypes.c_double * n)()
        w = (ctypes.c_double * n)()
        assert lib.bn_gauss_hermite(n, x, w) == 0
        xr, wr = np.polynomial.hermite.hermgauss(n)
        np.testing.assert_allclose(np.array(x), np.sqrt(2) * xr, rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(np.array(w), wr / np.sqrt(np.pi), rtol=1e-12, atol=1e-15)


def test_model_create_rejects_bad_arguments_without_gpu():
    from bayesnewton_gb300 import _lib
    lib = _built()
    h = ctypes.c_void_p()
    d = _lib.PriorDesc()
    lk = _lib.LikDesc()
    assert lib.bn_model_create(ctypes.byref(d), ctypes.byref(lk), 10, 1, 0, 0, ctypes.byref(h)) == _lib.ERR_ARG
    d.num_components = 1
    d.kind[0] = _lib.KIND_MATERN52
    d.size[0] = 3
    assert lib.bn_model_create(ctypes.byref(d), ctypes.byref(lk), 0, 1, 0, 0, ctypes.byref(h)) == _lib.ERR_ARG
    assert lib.bn_model_create(ctypes.byref(d), ctypes.byref(lk), 10, 1, 7, 0, ctypes.byref(h)) == _lib.ERR_ARG


def test_series_entry_points_reject_null_model_without_gpu():
    lib = _built()
    off = (ctypes.c_int64 * 2)(0, 10)
    one = (ctypes.c_double * 1)(1.0)
    kind = (ctypes.c_int32 * 1)(1)
    assert lib.bn_model_set_series(None, 1, off, one, one, kind, one) == -1
    out = (ctypes.c_double * 1)()
    assert lib.bn_model_series_energy(None, None, out) == -1


def test_series_batch_validates_before_touching_the_device():
    import pytest
    import bayesnewton_gb300 as bnx
    from bayesnewton_gb300.batch import MarkovSeriesBatch
    K, L = bnx.kernels, bnx.likelihoods
    x = [0.0, 1.0]
    with pytest.raises(ValueError):
        MarkovSeriesBatch([])
    with pytest.raises(ValueError):
        MarkovSeriesBatch([(K.Matern32(), L.Gaussian(), x, x), (K.Matern52(), L.Gaussian(), x, x)])
    with pytest.raises(NotImplementedError):
        MarkovSeriesBatch([(K.Sum([K.Matern32(), K.Matern12()]), L.Gaussian(), x, x)])
    with pytest.raises(NotImplementedError):
        MarkovSeriesBatch([(K.Matern32(), L.HeteroscedasticNoise("exp"), x, x)])
    with pytest.raises(ValueError):
        MarkovSeriesBatch([(K.Matern32(), L.Poisson(1.0), x, x), (K.Matern32(), L.Poisson(2.0), x, x)])


def test_library_prior_matrices_match_oracle():
    """Host-side prior matrices of the library's kernels (the values packed into
    bn_prior_desc and used by the generic expm path) against the oracle's
    (kernels.py:123-382, 1499-1663): Pinf, F and H agree, expm(F dt) equals the
    oracle's closed-form transition, and Pinf is the stationary solution of
    F Pinf + Pinf F^T + L Qc L^T = 0 (L the last state of each component, Qc > 0),
    which makes Q = Pinf - A Pinf A^T a covariance."""
    import numpy as np
    from scipy.linalg import expm

    import bayesnewton_gb300 as bnx
    from oracle import kernels as OK
    K = bnx.kernels
    pairs = [(K.Matern12(0.8, 1.3), OK.Matern12(0.8, 1.3)), (K.Matern32(1.2, 0.7), OK.Matern32(1.2, 0.7)),
             (K.Matern52(1.0, 2.0), OK.Matern52(1.0, 2.0)), (K.Matern72(0.9, 2.0), OK.Matern72(0.9, 2.0)),
             (K.Sum([K.Matern52(1.0, 1.5), K.Matern32(0.5, 4.0)]),
              OK.Sum([OK.Matern52(1.0, 1.5), OK.Matern32(0.5, 4.0)])),
             (K.Independent([K.Matern52(1.0, 2.0), K.Matern52(0.7, 5.0)]),
              OK.Independent([OK.Matern52(1.0, 2.0), OK.Matern52(0.7, 5.0)]))]
    for g, o in pairs:
        Pinf, F, H = g.stationary_covariance(), g.feedback_matrix(), g.measurement_model()
        np.testing.assert_allclose(Pinf, o.stationary_covariance(), rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(F, o.feedback_matrix(), rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(H, o.measurement_model(), rtol=0, atol=0)
        lyap = F @ Pinf + Pinf @ F.T
        last = np.cumsum([c.size for c in g.components()]) - 1
        assert np.all(lyap[last, last] < 0)
        lyap[last, last] = 0.0
        np.testing.assert_allclose(lyap, 0.0, atol=1e-11 * np.abs(Pinf).max())
        for dt in (0.0, 0.01, 0.37, 3.0):
            A = expm(F * dt)
            np.testing.assert_allclose(A, o.state_transition(dt), rtol=1e-10, atol=1e-12)
            Q = Pinf - A @ Pinf @ A.T
            assert np.linalg.eigvalsh(0.5 * (Q + Q.T)).min() > -1e-12 * np.abs(Pinf).max()
        d = g.desc()
        comps = g.components()
        assert d.num_components == len(comps)
        assert [d.size[i] for i in range(len(comps))] == [c.size for c in comps]


def test_library_likelihood_descriptors():
    """bn_lik_desc of each likelihood carries its kind, parameters and the
    reference's defaults (20 Gauss-Hermite points, the PSD fix on)."""
    import bayesnewton_gb300 as bnx
    from bayesnewton_gb300 import _lib
    L = bnx.likelihoods
    cases = [(L.Gaussian(0.3), _lib.LIK_GAUSSIAN), (L.Bernoulli("logit"), _lib.LIK_BERNOULLI_LOGIT),
             (L.Bernoulli("probit"), _lib.LIK_BERNOULLI_PROBIT), (L.Poisson(), _lib.LIK_POISSON_EXP),
             (L.HeteroscedasticNoise("exp"), _lib.LIK_HETERO_EXP),
             (L.HeteroscedasticNoise("softplus"), _lib.LIK_HETERO_SOFTPLUS)]
    for lik, kind in cases:
        d = lik.desc()
        assert d.kind == kind
        assert d.num_cub == 20 and d.ensure_psd == 1 and d.method == _lib.METHOD_VI
    assert abs(L.Gaussian(0.3).desc().variance - 0.3) < 1e-15
    d = L.Bernoulli("logit").desc(method=_lib.METHOD_EP, power=0.7)
    assert d.method == _lib.METHOD_EP and abs(d.power - 0.7) < 1e-15


def test_bounded_wait_probe_rejects_bad_arguments_without_gpu():
    """bn_bounded_wait_probe checks its poll limit and output pointer before it
    launches anything."""
    import ctypes as ct
    from bayesnewton_gb300 import _lib
    lib = _built()
    buf = (ct.c_int32 * 2)()
    assert lib.bn_bounded_wait_probe(None, 0, ct.addressof(buf)) == _lib.ERR_ARG
    assert lib.bn_bounded_wait_probe(None, (1 << 20) + 1, ct.addressof(buf)) == _lib.ERR_ARG
    assert lib.bn_bounded_wait_probe(None, 16, None) == _lib.ERR_ARG


def test_input_admin_sorts_and_rejects_corrupt_inputs():
    """utils.input_admin (utils.py:234-265) on the host: stable sort by time,
    dt = [0, diff(t)], Y reordered with X; mismatched lengths, empty inputs and
    non-finite times are rejected before any device work (NaN in Y stays a
    missing observation)."""
    import numpy as np
    import pytest
    import torch
    from bayesnewton_gb300.models import input_admin
    X = np.array([3.0, 1.0, 2.0, 1.0])
    Y = np.array([30.0, 10.0, np.nan, 11.0])
    t, y, dt, t64 = input_admin(X, Y, "cpu", torch.float32)
    assert t[:, 0].tolist() == [1.0, 1.0, 2.0, 3.0]
    assert np.isnan(y[2, 0].item()) and [y[0, 0].item(), y[1, 0].item(), y[3, 0].item()] == [10.0, 11.0, 30.0]
    assert dt.tolist() == [0.0, 0.0, 1.0, 1.0] and t64.dtype == torch.float64
    for bad_x, bad_y in [(X[:3], Y), (np.array([]), np.array([])), (np.array([1.0, np.nan]), np.array([1.0, 2.0])),
                         (np.array([1.0, np.inf]), np.array([1.0, 2.0]))]:
        with pytest.raises(ValueError):
            input_admin(bad_x, bad_y, "cpu", torch.float32)


def test_autotune_cache_file_round_trip(tmp_path):
    """The batch autotuner's cache file: keyed by GPU, kernel family, batch shape,
    dtype and method; a missing file reads as empty, entries are added or
    replaced, and a file that does not hold a JSON object is rejected."""
    import pytest
    import torch
    from bayesnewton_gb300.batch import autotune_key, load_autotune_cache, store_autotune_cache
    path = str(tmp_path / "tune.json")
    assert load_autotune_cache(path) == {}
    k1 = autotune_key("NVIDIA GB300", "Matern32", 4096, 32778340, torch.float32, "vi")
    k2 = autotune_key("NVIDIA GB300", "Matern32", 4096, 32778340, torch.float64, "vi")
    assert k1 != k2 and "float32" in k1 and "S=4096" in k1 and "N=32778340" in k1
    store_autotune_cache(path, k1, 16, {4: 3.1, 16: 2.9})
    store_autotune_cache(path, k2, 8, {8: 5.0})
    store_autotune_cache(path, k1, 32, {32: 2.5})
    data = load_autotune_cache(path)
    assert data[k1] == {"steps_per_thread": 32, "ms": {"32": 2.5}}
    assert data[k2]["steps_per_thread"] == 8
    (tmp_path / "bad.json").write_text("[1, 2]")
    with pytest.raises(ValueError):
        load_autotune_cache(str(tmp_path / "bad.json"))


def test_integration_xla_shim_compiles_and_links(tmp_path):
    """The XLA custom-call shim (integration/bn_xla.cc) compiles against
    include/bnx.h and links against libbnx.so (the jaxlib status symbol stays
    undefined, as it is resolved when jaxlib loads the shim)."""
    import shutil
    import subprocess
    import pytest
    from bayesnewton_gb300 import _lib
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    _built()
    src = os.path.join(ROOT, "integration", "bn_xla.cc")
    out = tmp_path / "libbn_xla.so"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-shared", "-fPIC", src, "-I", os.path.join(ROOT, "include"),
                        "-L", libdir, "-lbnx", "-Wl,-rpath," + libdir, "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def test_prior_descriptor_validation_without_gpu():
    """bn_model_create rejects malformed priors before any device work: no
    components, an unknown combine, a Matern kind whose size is not its order,
    a non-positive lengthscale and a state above 8."""
    from bayesnewton_gb300 import _lib
    lib = _built()
    lk = _lib.LikDesc()
    h = ctypes.c_void_p()

    def create(d):
        return lib.bn_model_create(ctypes.byref(d), ctypes.byref(lk), 10, 1, 0, 0, ctypes.byref(h))

    def m52():
        d = _lib.PriorDesc()
        d.num_components, d.combine = 1, _lib.COMBINE_SUM
        d.kind[0], d.size[0], d.variance[0], d.lengthscale[0] = _lib.KIND_MATERN52, 3, 1.0, 1.0
        return d

    d = m52()
    d.num_components = 0
    assert create(d) == _lib.ERR_ARG
    d = m52()
    d.combine = 7
    assert create(d) == _lib.ERR_ARG
    d = m52()
    d.size[0] = 2
    assert create(d) == _lib.ERR_ARG
    for ell in (0.0, -1.0, float("nan")):
        d = m52()
        d.lengthscale[0] = ell
        assert create(d) == _lib.ERR_ARG
    d = m52()
    d.num_components = 3
    for c in range(3):
        d.kind[c], d.size[c], d.variance[c], d.lengthscale[c] = _lib.KIND_MATERN52, 3, 1.0, 1.0
    assert create(d) == _lib.ERR_ARG  # state 9 > 8
    assert lib.bn_model_create(None, ctypes.byref(lk), 10, 1, 0, 0, ctypes.byref(h)) == _lib.ERR_ARG


def test_bench_reference_arm_json_contract():
    """bench.py --impl reference (the float64 port on the host cores) prints one
    JSON line with the benchmark contract's keys, on a small series."""
    import json
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--num-data", "20000",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["higher_is_better"] is False and d["value"] > 0
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_bench_algorithmic_bytes_follow_the_step_formula():
    """bench.py's algorithmic bytes per time point: 4 [1 + p + 2s + s + 2(d + d(d+1)/2)]
    with s = p + p(p+1)/2 gives 104 B (plain, d = 3), 192 B (long series, d = 5),
    72 B (many series, d = 2) and 288 B (two latents, d = 6, p = 2)."""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.step_bytes(3) == 104 and bench.step_bytes(5) == 192 and bench.step_bytes(2) == 72
    assert bench.step_bytes(6, p=2) == 288
    kb = bench.kernel_bytes(5)
    assert kb["filter_reduce"] == 32 and kb["site_tail"] == 32
    assert kb["filter_rerun"] == 4 * (4 + 20) and kb["smoother_rerun"] == 4 * (20 + 2)


def test_noalloc_filter_rejects_unsupported_priors_without_gpu():
    """bn_kalman_filter_noalloc accepts a single Matern or Sum(Matern52, Matern32)
    in that order only: Sum(Matern32, Matern52), a three-component sum and a
    product are rejected with BN_ERR_UNSUPPORTED, and malformed descriptors with
    BN_ERR_ARG, before any device work (the pointers are never read)."""
    from bayesnewton_gb300 import _lib
    lib = _built()
    f = lib.bn_kalman_filter_noalloc
    vp = ctypes.c_void_p
    f.argtypes = [ctypes.POINTER(_lib.PriorDesc), ctypes.c_int64, vp, ctypes.c_int32, vp, vp, vp, vp, vp, vp, vp, vp]
    f.restype = ctypes.c_int
    dummy = ctypes.c_void_p(16)

    def call(d):
        return f(ctypes.byref(d), 1000, None, 0, dummy, dummy, dummy, None, dummy, dummy, None, None)

    def prior(kinds, combine=_lib.COMBINE_SUM):
        d = _lib.PriorDesc()
        d.num_components, d.combine = len(kinds), combine
        for c, k in enumerate(kinds):
            d.kind[c], d.size[c], d.variance[c], d.lengthscale[c] = k, k, 1.0, 1.0
        return d

    M32, M52 = _lib.KIND_MATERN32, _lib.KIND_MATERN52
    assert call(prior([M32, M52])) == _lib.ERR_UNSUPPORTED
    assert call(prior([M52, M32, M32])) == _lib.ERR_UNSUPPORTED
    assert call(prior([M52, M32], combine=_lib.COMBINE_SUM + 1)) == _lib.ERR_UNSUPPORTED
    d = prior([M52, M32])
    d.lengthscale[1] = 0.0
    assert call(d) == _lib.ERR_ARG
    assert f(None, 1000, None, 0, dummy, dummy, dummy, None, dummy, dummy, None, None) == _lib.ERR_ARG


def _exact_matern_q(S, var, ell, dt):
    """Q = Pinf - A Pinf A^T of a Matern block in 60-digit arithmetic (mpmath), with
    the reference's companion-form feedback and stationary covariance
    (kernels.py:123-382) written as exact rationals times powers of lam."""
    from fractions import Fraction as Fr
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 60
    lam = mp.sqrt(2 * S - 1) / mp.mpf(ell)
    binom = [[1], [1, 1], [1, 2, 1], [1, 3, 3, 1], [1, 4, 6, 4, 1]][S]
    F = mp.zeros(S, S)
    for i in range(S - 1):
        F[i, i + 1] = 1
    for k in range(S):
        F[S - 1, k] = -binom[k] * lam ** (S - k)
    pt = {1: {}, 2: {}, 3: {(1, 1): Fr(1, 3), (0, 2): Fr(-1, 3)},
          4: {(1, 1): Fr(1, 5), (2, 2): Fr(1, 5), (0, 2): Fr(-1, 5), (1, 3): Fr(-1, 5)}}[S]
    Pinf = mp.zeros(S, S)
    for i in range(S):
        for j in range(S):
            r = Fr(1) if i == j else Fr(0)
            r = pt.get((min(i, j), max(i, j)), r)
            Pinf[i, j] = mp.mpf(var) * lam ** (i + j) * mp.mpf(r.numerator) / r.denominator
    A = mp.expm(F * mp.mpf(dt))
    Q = Pinf - A * Pinf * A.T
    return np.array([[float(Q[i, j]) for j in range(S)] for i in range(S)]), float(lam)


def test_float32_process_noise_keeps_its_digits():
    """The float32 process noise the kernels form for a Matern block (exported as
    bn_matern_process_noise) against Q = Pinf - A Pinf A^T in 60-digit arithmetic,
    for Matern12/32/52/72 over lam dt in [1e-4, 25]: every entry within 1e-6 of
    sqrt(Q_ii Q_jj).  The direct float32 form Pinf - A Pinf A^T, which the float32
    path used to take, is off by more than its own size there (e.g. Matern52 at
    lam dt = 0.01), which is what made float32 posteriors drift at dense inputs."""
    from bayesnewton_gb300 import _lib
    lib = _built()
    f = lib.bn_matern_process_noise
    f.argtypes = [ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                  ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    f.restype = ctypes.c_int
    var, ell = 1.7, 0.8
    worst = {}
    for S in (1, 2, 3, 4):
        lam = np.sqrt(2 * S - 1) / ell
        for x in np.logspace(-4, np.log10(25.0), 30):
            dt = x / lam
            a = (ctypes.c_float * (S * S))()
            q = (ctypes.c_float * (S * S))()
            assert f(S, var, ell, dt, a, q) == 0
            Q32 = np.array(q[:], dtype=np.float64).reshape(S, S)
            Qx, _ = _exact_matern_q(S, var, ell, dt)
            d = np.sqrt(np.abs(np.diag(Qx)))
            err = float(np.max(np.abs(Q32 - Qx) / np.outer(d, d)))
            worst[S] = max(worst.get(S, 0.0), err)
    assert max(worst.values()) < 1e-6, worst
    # the direct form in float32 at Matern52, lam dt = 0.01
    S, x = 3, 0.01
    lam = np.sqrt(5.0) / ell
    a = (ctypes.c_float * 9)()
    q = (ctypes.c_float * 9)()
    assert f(S, var, ell, x / lam, a, q) == 0
    A = np.array(a[:], dtype=np.float32).reshape(3, 3)
    Qx, _ = _exact_matern_q(S, var, ell, x / lam)
    l2 = lam * lam
    Pinf = (var * np.array([[1, 0, -l2 / 3], [0, l2 / 3, 0], [-l2 / 3, 0, l2 * l2]])).astype(np.float32)
    direct = (Pinf - A @ Pinf @ A.T).astype(np.float64)
    assert abs(direct[0, 0] - Qx[0, 0]) > abs(Qx[0, 0])
    # argument checks
    assert f(5, var, ell, 0.1, a, q) == _lib.ERR_ARG
    assert f(2, var, -1.0, 0.1, a, q) == _lib.ERR_ARG


def test_dense_inverse_rejects_bad_arguments_without_gpu():
    """bn_dense_inverse checks its engine, sizes and pointer before any device work:
    an unknown engine, an empty batch, a null matrix and, for the register-resident
    engines (1, 2), n above 200 return BN_ERR_ARG."""
    lib = _built()
    f = lib.bn_dense_inverse
    vp = ctypes.c_void_p
    f.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, vp, vp, vp]
    f.restype = ctypes.c_int
    dummy = vp(16)
    err_arg = -1
    assert f(None, 3, 1, 8, dummy, None, None) == err_arg
    assert f(None, -1, 1, 8, dummy, None, None) == err_arg
    assert f(None, 1, 0, 8, dummy, None, None) == err_arg
    assert f(None, 1, 1, 0, dummy, None, None) == err_arg
    assert f(None, 1, 1, 8, None, None, None) == err_arg
    assert f(None, 1, 1, 201, dummy, None, None) == err_arg
    assert f(None, 2, 1, 201, dummy, None, None) == err_arg
