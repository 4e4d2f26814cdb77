"""GB300-native Markov-GP inference step with the interface of bayesnewton.

Modules mirror the reference package: ``kernels``, ``likelihoods``, ``cubature``,
``ops`` (kalman_filter / rauch_tung_striebel_smoother) and ``models``
(MarkovVariationalGP, MarkovNewtonGP, MarkovExpectationPropagationGP).  Compute
runs in libbnx.so (hand-written CUDA for sm_103a, C ABI in include/bnx.h).
"""
from . import _lib, batch, cubature, infinite_horizon, kernels, likelihoods, models, ops, spatiotemporal, surrogate  # noqa: F401


def build_model(model, inf, name="GPModel"):
    """Compose a model class from a base and an inference mixin (the reference's
    bayesnewton/__init__.py:13-14).  Here the inference method is a class
    attribute of the model classes, so the composition picks it up from `inf`."""
    return type(name, (model,), {"_method": getattr(inf, "_method", _lib.METHOD_VI)})


class VariationalInference:
    _method = _lib.METHOD_VI


class Newton:
    _method = _lib.METHOD_NEWTON


class ExpectationPropagation:
    _method = _lib.METHOD_EP
