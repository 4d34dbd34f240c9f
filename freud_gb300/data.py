"""Synthetic systems, API-compatible with the parts of freud.data used on this
path (freud/data.py:44-153, 350-376): make_random_system and UnitCell lattices."""

import numpy as np

from .box import Box


def make_random_system(box_size, num_points, is2D=False, seed=None):
    """Uniform random points in a cubic (or square) box (freud/data.py:350-376)."""
    rs = np.random.RandomState(seed)
    fractional_coords = rs.random_sample((num_points, 3))
    if is2D:
        box = Box.square(box_size)
        fractional_coords[:, 2] = 0
    else:
        box = Box.cube(box_size)
    points = box.make_absolute(fractional_coords)
    return box, points


class UnitCell:
    """A unit cell: a box and fractional basis positions."""

    def __init__(self, box, basis_positions=((0, 0, 0),)):
        self._box = Box.from_box(box)
        self._basis_positions = np.asarray(basis_positions, dtype=np.float64)

    @property
    def box(self):
        return self._box

    @property
    def basis_positions(self):
        return self._basis_positions

    @property
    def dimensions(self):
        return self._box.dimensions

    def generate_system(self, num_replicas=1, scale=1.0, sigma_noise=0.0, seed=None):
        """Replicate the cell, scale it, add Gaussian noise and wrap into the box.
        Positions are ordered basis-major (like numpy.repeat over the basis)."""
        try:
            nx, ny, nz = num_replicas
        except TypeError:
            nx = ny = num_replicas
            nz = 1 if self.box.is2D else num_replicas
        if not all(int(n) == n and n > 0 for n in (nx, ny, nz)):
            raise ValueError("The number of replicas must be a positive integer in each dimension.")
        if self.box.is2D and nz != 1:
            raise ValueError("The number of replicas in z must be 1 for a 2D unit cell.")
        a1, a2, a3 = self.box.v1, self.box.v2, (self.box.v3 if not self.box.is2D else np.zeros(3))
        gx, gy, gz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        shifts = (gx.reshape(-1, 1) * a1 + gy.reshape(-1, 1) * a2 + gz.reshape(-1, 1) * a3)
        basis_abs = self.box.make_absolute(self.basis_positions).astype(np.float64)
        positions = (basis_abs[:, None, :] + shifts[None, :, :]).reshape(-1, 3)
        box = Box(self.box.Lx * nx, self.box.Ly * ny, self.box.Lz * nz, self.box.xy, self.box.xz, self.box.yz,
                  self.box.is2D)
        # centre the replicated lattice in the box
        positions = positions - (np.array([nx, ny, nz]) - 1) / 2.0 * np.array([self.box.Lx, self.box.Ly, self.box.Lz])
        box = box * scale
        positions = positions * scale
        positions = box.wrap(positions.astype(np.float32))
        if sigma_noise != 0:
            rs = np.random.RandomState(seed)
            var = sigma_noise * sigma_noise
            cov = np.diag([var, var, var if self.dimensions == 3 else 0])
            positions = positions + rs.multivariate_normal([0, 0, 0], cov, size=positions.shape[:-1])
        positions = box.wrap(np.asarray(positions, dtype=np.float32))
        return box, positions

    @classmethod
    def fcc(cls):
        return cls(Box.cube(1), [[0.25, 0.25, 0.25], [0.75, 0.75, 0.25], [0.75, 0.25, 0.75], [0.25, 0.75, 0.75]])

    @classmethod
    def bcc(cls):
        return cls(Box.cube(1), [[0.25, 0.25, 0.25], [0.75, 0.75, 0.75]])

    @classmethod
    def sc(cls):
        return cls(Box.cube(1), [[0.5, 0.5, 0.5]])

    @classmethod
    def square(cls):
        return cls(Box.square(1), [[0.5, 0.5, 0]])

    @classmethod
    def hex(cls):
        return cls(Box(1, np.sqrt(3), is2D=True), [[0, 0, 0], [0.5, 0.5, 0]])
