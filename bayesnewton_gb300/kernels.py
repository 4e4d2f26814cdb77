"""State-space GP priors (the interface of bayesnewton/kernels.py).

A kernel here is a small host-side description (hyperparameters and block
structure) that the CUDA library turns into its device transition A(dt), Pinf and
H.  Supported: Matern12/32/52/72 (kernels.py:123-382), Sum (:1624-1663),
Independent (:1499-1616) and a generic StateSpace prior given by its feedback
matrix F and stationary covariance Pinf, whose transition is expm(F dt)
(the generic Kernel.state_transition, kernels.py:63-67).

Changing a hyperparameter bumps a version counter that models watch, so the next
inference() refreshes the posterior under the new prior as the reference does.
"""
import ctypes
import math

import numpy as np

from . import _lib


class Kernel:
    _params = ()

    def __init__(self):
        object.__setattr__(self, "_version", 0)

    def __setattr__(self, name, value):
        object.__setattr__(self, name, value)
        if name in self._params:
            object.__setattr__(self, "_version", self._version + 1)

    @property
    def version(self):
        return self._version

    def components(self):
        return [self]

    def combine(self):
        return _lib.COMBINE_SUM

    @property
    def state_dim(self):
        return sum(c.size for c in self.components())

    def stationary_covariance(self):
        blocks = [c._pinf() for c in self.components()]
        return _block_diag(blocks)

    def feedback_matrix(self):
        return _block_diag([c._feedback() for c in self.components()])

    def measurement_model(self):
        comps = self.components()
        D = self.state_dim
        if self.combine() == _lib.COMBINE_SUM:
            H = np.zeros([1, D])
            o = 0
            for c in comps:
                H[0, o] = 1.0
                o += c.size
        else:
            H = np.zeros([len(comps), D])
            o = 0
            for i, c in enumerate(comps):
                H[i, o] = 1.0
                o += c.size
        return H

    def desc(self):
        """The bn_prior_desc of this prior."""
        d = _lib.PriorDesc()
        comps = self.components()
        if len(comps) > _lib.MAX_COMPONENTS or self.state_dim > _lib.MAX_STATE:
            raise ValueError("prior too large for the small-state path (D <= %d)" % _lib.MAX_STATE)
        d.num_components = len(comps)
        d.combine = self.combine()
        o = 0
        for i, c in enumerate(comps):
            d.kind[i] = c.kind
            d.size[i] = c.size
            d.variance[i] = float(getattr(c, "variance", 1.0))
            d.lengthscale[i] = float(getattr(c, "lengthscale", 1.0))
            if c.kind == _lib.KIND_FEEDBACK:
                F, Pi = c._feedback(), c._pinf()
                for a in range(c.size):
                    for b in range(c.size):
                        d.feedback[(o + a) * _lib.MAX_STATE + o + b] = float(F[a, b])
                        d.pinf[(o + a) * _lib.MAX_STATE + o + b] = float(Pi[a, b])
            o += c.size
        return d


def _block_diag(blocks):
    n = sum(b.shape[0] for b in blocks)
    out = np.zeros([n, n])
    o = 0
    for b in blocks:
        s = b.shape[0]
        out[o:o + s, o:o + s] = b
        o += s
    return out


class StationaryKernel(Kernel):
    _params = ("variance", "lengthscale")

    def __init__(self, variance=1.0, lengthscale=1.0, fix_variance=False, fix_lengthscale=False):
        super().__init__()
        self.variance = float(variance)
        self.lengthscale = float(lengthscale)
        self.fix_variance = fix_variance
        self.fix_lengthscale = fix_lengthscale


class Matern12(StationaryKernel):
    kind, size = _lib.KIND_MATERN12, 1

    def _pinf(self):
        return np.array([[self.variance]])

    def _feedback(self):
        return np.array([[-1.0 / self.lengthscale]])


class Matern32(StationaryKernel):
    kind, size = _lib.KIND_MATERN32, 2

    def _pinf(self):
        return np.array([[self.variance, 0.0], [0.0, 3.0 * self.variance / self.lengthscale ** 2]])

    def _feedback(self):
        lam = math.sqrt(3.0) / self.lengthscale
        return np.array([[0.0, 1.0], [-lam ** 2, -2 * lam]])


class Matern52(StationaryKernel):
    kind, size = _lib.KIND_MATERN52, 3

    def _pinf(self):
        v, l = self.variance, self.lengthscale
        k = 5.0 / 3.0 * v / l ** 2
        return np.array([[v, 0.0, -k], [0.0, k, 0.0], [-k, 0.0, 25.0 * v / l ** 4]])

    def _feedback(self):
        lam = math.sqrt(5.0) / self.lengthscale
        return np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [-lam ** 3, -3.0 * lam ** 2, -3.0 * lam]])


class Matern72(StationaryKernel):
    kind, size = _lib.KIND_MATERN72, 4

    def _pinf(self):
        v, l = self.variance, self.lengthscale
        k, k2 = 7.0 / 5.0 * v / l ** 2, 9.8 * v / l ** 4
        return np.array([[v, 0.0, -k, 0.0], [0.0, k, 0.0, -k2], [-k, 0.0, k2, 0.0],
                         [0.0, -k2, 0.0, 343.0 * v / l ** 6]])

    def _feedback(self):
        lam = math.sqrt(7.0) / self.lengthscale
        return np.array([[0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0],
                         [-lam ** 4, -4.0 * lam ** 3, -6.0 * lam ** 2, -4.0 * lam]])


Exponential = Matern12


class StateSpace(Kernel):
    """A prior given by (F, Pinf): transition expm(F dt), H = [1, 0, ...]."""
    kind = _lib.KIND_FEEDBACK
    _params = ("F", "Pinf")

    def __init__(self, F, Pinf):
        super().__init__()
        self.F = np.asarray(F, dtype=np.float64)
        self.Pinf = np.asarray(Pinf, dtype=np.float64)
        self.size = self.F.shape[0]

    def _pinf(self):
        return self.Pinf

    def _feedback(self):
        return self.F


class Independent(Kernel):
    """Stacked independent priors, one latent each (kernels.py:1499-1616)."""

    def __init__(self, kernels):
        super().__init__()
        self.kernels = list(kernels)
        self.num_kernels = len(self.kernels)

    @property
    def version(self):
        return sum(k.version for k in self.kernels)

    def components(self):
        out = []
        for k in self.kernels:
            out.extend(k.components())
        return out

    def combine(self):
        return _lib.COMBINE_INDEPENDENT


Separate = Stack = Independent


class Sum(Independent):
    """Sum of priors: one latent, H = [H_1, H_2, ...] (kernels.py:1624-1663)."""

    def combine(self):
        return _lib.COMBINE_SUM


class SpatioTemporalKernel(Kernel):
    """Separable spatio-temporal prior, Markov in time and sparse in space
    (kernels.py:385-586): a temporal Matern12/32/52 kernel for each of the M
    spatial inducing inputs z [M, D], a spatial Matern12/32/52 kernel, and the
    'Full' (or 'FIC', whose diagonal is the same) or 'DTC' spatial conditional.
    Only the sparse form is supported; z is fixed (opt_z=False)."""

    def __init__(self, temporal_kernel, spatial_kernel, z=None, conditional=None, sparse=True, opt_z=False,
                 spatial_dims=None):
        super().__init__()
        if not sparse:
            raise NotImplementedError("only the sparse spatio-temporal form is supported")
        if opt_z:
            raise NotImplementedError("optimising z is not on this path")
        for k in (temporal_kernel, spatial_kernel):
            if type(k) not in (Matern12, Matern32, Matern52):
                raise NotImplementedError("temporal and spatial kernels must be Matern12/32/52")
        if z is None:
            if spatial_dims == 1:
                z = np.linspace(-3.0, 3.0, num=15)
            elif spatial_dims == 2:
                z1 = np.linspace(-3.0, 3.0, num=5)
                za, zb = np.meshgrid(z1, z1)
                z = np.hstack((za.reshape(-1, 1), zb.reshape(-1, 1)))
            else:
                raise NotImplementedError("please provide an initialisation for inducing inputs z")
        z = np.asarray(z, dtype=np.float64)
        if z.ndim < 2:
            z = z[:, None]
        conditional = "Full" if conditional is None else conditional
        if conditional.lower() in ("full", "fic", "fitc"):
            self.conditional = 0
        elif conditional.lower() == "dtc":
            self.conditional = 1
        else:
            raise NotImplementedError("conditional method not recognised")
        self.temporal_kernel = temporal_kernel
        self.spatial_kernel = spatial_kernel
        self.z = np.ascontiguousarray(z)
        self.M = z.shape[0]

    @property
    def version(self):
        return self.temporal_kernel.version + self.spatial_kernel.version + self._version

    @property
    def state_dim(self):
        return self.M * self.temporal_kernel.size

    @property
    def variance(self):
        return self.temporal_kernel.variance

    @property
    def temporal_lengthscale(self):
        return self.temporal_kernel.lengthscale

    @property
    def spatial_lengthscale(self):
        return self.spatial_kernel.lengthscale

    def st_desc(self):
        """The bn_st_desc of this prior (keeps z alive on self)."""
        d = _lib.StDesc()
        d.temporal_kind = self.temporal_kernel.kind
        d.temporal_variance = self.temporal_kernel.variance
        d.temporal_lengthscale = self.temporal_kernel.lengthscale
        d.spatial_kind = self.spatial_kernel.kind
        d.spatial_variance = self.spatial_kernel.variance
        d.spatial_lengthscale = self.spatial_kernel.lengthscale
        d.num_inducing = self.M
        d.spatial_dim = self.z.shape[1]
        d.z = self.z.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.conditional = self.conditional
        return d


class SpatioTemporalMatern12(SpatioTemporalKernel):
    """kernels.py:588-609."""

    def __init__(self, variance=1.0, lengthscale_time=1.0, lengthscale_space=1.0, z=None, sparse=True,
                 opt_z=False, conditional=None):
        super().__init__(Matern12(variance, lengthscale_time), Matern12(1.0, lengthscale_space), z=z,
                         conditional=conditional, sparse=sparse, opt_z=opt_z)


class SpatioTemporalMatern32(SpatioTemporalKernel):
    """kernels.py:612-633."""

    def __init__(self, variance=1.0, lengthscale_time=1.0, lengthscale_space=1.0, z=None, sparse=True,
                 opt_z=False, conditional=None):
        super().__init__(Matern32(variance, lengthscale_time), Matern32(1.0, lengthscale_space), z=z,
                         conditional=conditional, sparse=sparse, opt_z=opt_z)


class SpatioTemporalMatern52(SpatioTemporalKernel):
    """kernels.py:639-660."""

    def __init__(self, variance=1.0, lengthscale_time=1.0, lengthscale_space=1.0, z=None, sparse=True,
                 opt_z=False, conditional=None):
        super().__init__(Matern52(variance, lengthscale_time), Matern52(1.0, lengthscale_space), z=z,
                         conditional=conditional, sparse=sparse, opt_z=opt_z)
