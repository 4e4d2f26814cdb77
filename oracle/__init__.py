"""Oracle: a float64 CPU restatement of BayesNewton's Markov-GP inference step.

TEST INFRASTRUCTURE ONLY.  Nothing in the product path (the ``bayesnewton_gb300``
package and its CUDA library) may import, call or link anything in this package.
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, and only as the parity reference / the timed CPU baseline.

Contents
--------
- ``kernels``      Matern12/32/52/72 SDE priors, Sum, Independent and a generic
                   feedback-matrix kernel whose transition is ``expm(F dt)``
                   (bayesnewton/kernels.py:63-67, 123-382, 1499-1663).
- ``likelihoods``  Gaussian, Bernoulli (logit / probit), Poisson (exp link) and
                   HeteroscedasticNoise (bayesnewton/likelihoods.py:326-412,
                   613-664, 684-1008, 1244-1281).
- ``cubature``     Gauss-Hermite rules and the cubature site expectations
                   (bayesnewton/cubature.py:56-84, 198-246, 310-371).
- ``ops``          sequential and parallel (associative-scan) Kalman filter and
                   RTS smoother (bayesnewton/ops.py:149-380).
- ``models``       Markov GP with VI / Newton / EP site updates and energies, and
                   the dense-GP model used by the reference's consistency tests
                   (bayesnewton/basemodels.py:52-378, 625-764;
                   bayesnewton/inference.py:21-325).
- ``cpu_ref.cpp``  the same sequential arithmetic in C++ (float64), used for large
                   N in tests and as the timed CPU baseline (``kind: "port"``).

Parity pinning: the reference cannot run here (no JAX).  The oracle is pinned
by restating the reference's own known-answer and consistency tests
(tests/test_vs_exact_marg_lik.py:41-59, tests/test_gp_vs_markovgp_reg.py:48-138,
tests/test_gp_vs_markovgp_class.py:38-124) on seeded data; see tests/test_oracle_*.py.
Its outputs on fourteen seeded cases are committed as golden fixtures
(tests/golden/*.npz, written by tests/golden/make_golden.py together with dense-GP
and exact-GP values that do not use the state-space code; tests/test_golden.py).

The parallel filter follows the reference's combine (ops.py:203-219, through
inv(C1)) by default; ``ops.kalman_filter(..., stable=True)`` and
``models.MarkovGP(..., stable=True)`` use the (I + C1 J2)^-1 form instead, which
holds where C1 is singular to working precision (inputs much closer than the
lengthscale) and equals the sequential filter there.
"""
