"""Kernel / likelihood specifications of the golden fixtures, and their
construction as oracle objects and as library objects.

A kernel spec is ``["Matern52", variance, lengthscale]`` (any Matern order) or
``["Sum" | "Independent", spec, spec, ...]``; a likelihood spec is
``["Gaussian", noise]``, ``["Bernoulli", link]``, ``["Poisson"]`` or
``["HeteroscedasticNoise", link]``."""


def _kernel(mod, spec):
    if spec[0] in ("Sum", "Independent"):
        return getattr(mod, spec[0])([_kernel(mod, s) for s in spec[1:]])
    return getattr(mod, spec[0])(float(spec[1]), float(spec[2]))


def _likelihood(mod, spec):
    return getattr(mod, spec[0])(*spec[1:])


def oracle_kernel(spec):
    from oracle import kernels
    return _kernel(kernels, spec)


def oracle_likelihood(spec):
    from oracle import likelihoods
    return _likelihood(likelihoods, spec)


def oracle_st_kernel(spec, z):
    from oracle.spatiotemporal import SpatioTemporalKernel
    return SpatioTemporalKernel(oracle_kernel(spec["temporal"]), oracle_kernel(spec["spatial"]), z)


def library_kernel(spec):
    import bayesnewton_gb300 as bnx
    return _kernel(bnx.kernels, spec)


def library_likelihood(spec):
    import bayesnewton_gb300 as bnx
    return _likelihood(bnx.likelihoods, spec)


def library_st_kernel(spec, z):
    import bayesnewton_gb300 as bnx
    return bnx.kernels.SpatioTemporalKernel(library_kernel(spec["temporal"]), library_kernel(spec["spatial"]),
                                            z=z)
