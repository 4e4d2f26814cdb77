"""Cubature rule descriptors (bayesnewton/cubature.py:31-39).

The nodes and weights themselves are generated inside the CUDA library; this
object only carries the number of points per latent."""


class GaussHermite:
    def __init__(self, dim=None, num_cub_points=20):
        if num_cub_points > 32:
            raise ValueError("at most 32 Gauss-Hermite points per latent")
        self.dim = dim
        self.num_cub_points = int(num_cub_points)
