"""Periodic simulation box, API-compatible with freud.box (freud/box.py:28-981).

The arithmetic (fractional/absolute conversion, wrap, nearest-plane distances,
lattice vectors) is float32 in the operation order of freud/box/Box.h:101-518,
so vectors produced here are bit-identical to the reference's.
"""

import warnings

import numpy as np

_f32 = np.float32


class Box:
    """A triclinic box centred at the origin, spanning [-L/2, L/2) in each direction.

    Args:
        Lx, Ly (float): box lengths; Lz (float, optional): 0 for 2D boxes.
        xy, xz, yz (float, optional): tilt factors.
        is2D (bool, optional): inferred from ``Lz == 0`` when None.
    """

    def __init__(self, Lx, Ly, Lz=0, xy=0, xz=0, yz=0, is2D=None):
        if is2D is None:
            is2D = Lz == 0
        if is2D:
            if not (Lx and Ly):
                raise ValueError("Lx and Ly must be nonzero for 2D boxes.")
            if Lz != 0 or xz != 0 or yz != 0:
                warnings.warn("Specifying z-dimensions in a 2-dimensional box has no effect!", stacklevel=2)
        elif not (Lx and Ly and Lz):
            raise ValueError("Lx, Ly, and Lz must be nonzero for 3D boxes.")
        self._is2D = bool(is2D)
        self._set_L(Lx, Ly, Lz)
        self._xy, self._xz, self._yz = _f32(xy), _f32(xz), _f32(yz)
        self._periodic = [True, True, True]

    # -- construction helpers ---------------------------------------------------
    def _set_L(self, Lx, Ly, Lz):
        # Box::setL (Box.h:101-116)
        if self._is2D:
            self._L = np.array([Lx, Ly, 0], dtype=_f32)
        else:
            self._L = np.array([Lx, Ly, Lz], dtype=_f32)
        self._hi = self._L / _f32(2.0)
        self._lo = -self._hi

    @classmethod
    def cube(cls, L=None):
        if L is None:
            raise TypeError("cube() missing 1 required positional argument: 'L'")
        return cls(Lx=L, Ly=L, Lz=L, xy=0, xz=0, yz=0, is2D=False)

    @classmethod
    def square(cls, L=None):
        if L is None:
            raise TypeError("square() missing 1 required positional argument: 'L'")
        return cls(Lx=L, Ly=L, Lz=0, xy=0, xz=0, yz=0, is2D=True)

    @classmethod
    def from_matrix(cls, box_matrix, dimensions=None):
        # float32 first, as freud does (freud/box.py:862): the derived lengths and
        # tilts then round exactly as the reference's
        m = np.asarray(box_matrix, dtype=np.float32)
        v0, v1, v2 = m[:, 0], m[:, 1], m[:, 2]
        Lx = np.sqrt(np.dot(v0, v0))
        a2x = np.dot(v0, v1) / Lx
        Ly = np.sqrt(np.dot(v1, v1) - a2x * a2x)
        xy = a2x / Ly
        v0xv1 = np.cross(v0, v1)
        v0xv1mag = np.sqrt(np.dot(v0xv1, v0xv1))
        Lz = np.dot(v2, v0xv1) / v0xv1mag
        if Lz != 0:
            a3x = np.dot(v0, v2) / Lx
            xz = a3x / Lz
            yz = (np.dot(v1, v2) - a2x * a3x) / (Ly * Lz)
        else:
            xz = yz = 0
        if dimensions is None:
            dimensions = 2 if Lz == 0 else 3
        return cls(Lx=Lx, Ly=Ly, Lz=Lz, xy=xy, xz=xz, yz=yz, is2D=dimensions == 2)

    @classmethod
    def from_box(cls, box, dimensions=None):
        """Initialise from a Box, a dict, a sequence of up to six numbers
        (Lx, Ly, Lz, xy, xz, yz), a 3x3 matrix, or an object with those attributes."""
        if np.asarray(box).shape == (3, 3):
            return cls.from_matrix(box, dimensions=dimensions)
        if isinstance(box, Box):
            b = Box(box.Lx, box.Ly, box.Lz, box.xy, box.xz, box.yz, box.is2D)
            b.periodic = box.periodic
            return b
        is2D = None
        if isinstance(box, dict):
            Lx, Ly = box["Lx"], box["Ly"]
            Lz = box.get("Lz", 0)
            xy, xz, yz = box.get("xy", 0), box.get("xz", 0), box.get("yz", 0)
            if "dimensions" in box and box["dimensions"] is not None:
                is2D = box["dimensions"] == 2
        elif all(hasattr(box, a) for a in ("Lx", "Ly")):
            Lx, Ly = box.Lx, box.Ly
            Lz = getattr(box, "Lz", 0)
            xy, xz, yz = getattr(box, "xy", 0), getattr(box, "xz", 0), getattr(box, "yz", 0)
            if hasattr(box, "dimensions"):
                is2D = box.dimensions == 2
        else:
            try:
                seq = [float(x) for x in np.asarray(box, dtype=np.float64).ravel()]
            except (TypeError, ValueError) as e:
                raise ValueError("Supplied box cannot be converted to type freud.box.Box.") from e
            if len(seq) not in (2, 3, 6):
                raise ValueError("List-like objects must have length 2, 3, or 6 to be converted to freud.box.Box.")
            seq = seq + [0] * (6 - len(seq))
            Lx, Ly, Lz, xy, xz, yz = seq
        if dimensions is not None:
            is2D = dimensions == 2
        if is2D is None:
            is2D = Lz == 0
        return cls(Lx=Lx, Ly=Ly, Lz=Lz, xy=xy, xz=xz, yz=yz, is2D=is2D)

    # -- properties ---------------------------------------------------------------
    @property
    def L(self):
        return np.array(self._L, dtype=np.float64)

    @L.setter
    def L(self, value):
        try:
            if len(value) != 3:
                raise ValueError("setL must be called with a scalar or a list of length 3.")
        except TypeError:
            value = [value, value, 0 if self.is2D else value]
        if self.is2D and value[2] != 0:
            warnings.warn("Specifying z-dimensions in a 2-dimensional box has no effect!", stacklevel=2)
        self._set_L(*value)

    @property
    def Lx(self):
        return float(self._L[0])

    @Lx.setter
    def Lx(self, value):
        self._set_L(value, self._L[1], self._L[2])

    @property
    def Ly(self):
        return float(self._L[1])

    @Ly.setter
    def Ly(self, value):
        self._set_L(self._L[0], value, self._L[2])

    @property
    def Lz(self):
        return float(self._L[2])

    @Lz.setter
    def Lz(self, value):
        self._set_L(self._L[0], self._L[1], value)

    @property
    def xy(self):
        return float(self._xy)

    @xy.setter
    def xy(self, value):
        self._xy = _f32(value)

    @property
    def xz(self):
        return float(self._xz)

    @xz.setter
    def xz(self, value):
        self._xz = _f32(value)

    @property
    def yz(self):
        return float(self._yz)

    @yz.setter
    def yz(self, value):
        self._yz = _f32(value)

    @property
    def dimensions(self):
        return 2 if self.is2D else 3

    @dimensions.setter
    def dimensions(self, value):
        assert value == 2 or value == 3
        self._is2D = value == 2
        self._set_L(self._L[0], self._L[1], self._L[2])

    @property
    def is2D(self):
        return self._is2D

    @property
    def L_inv(self):
        with np.errstate(divide="ignore"):
            inv = _f32(1) / self._L
        if self.is2D:
            inv[2] = 0
        return np.array(inv, dtype=np.float64)

    @property
    def volume(self):
        if self.is2D:
            return float(self._L[0] * self._L[1])
        return float(self._L[0] * self._L[1] * self._L[2])

    @property
    def periodic(self):
        return np.array(self._periodic, dtype=bool)

    @periodic.setter
    def periodic(self, periodic):
        periodic = np.asarray(periodic, dtype=bool).ravel()
        if periodic.size == 1:
            periodic = np.repeat(periodic, 3)
        self._periodic = [bool(p) for p in periodic]

    @property
    def periodic_x(self):
        return self._periodic[0]

    @periodic_x.setter
    def periodic_x(self, v):
        self._periodic[0] = bool(v)

    @property
    def periodic_y(self):
        return self._periodic[1]

    @periodic_y.setter
    def periodic_y(self, v):
        self._periodic[1] = bool(v)

    @property
    def periodic_z(self):
        return self._periodic[2]

    @periodic_z.setter
    def periodic_z(self, v):
        self._periodic[2] = bool(v)

    @property
    def cubic(self):
        return (not self.is2D and self.Lx == self.Ly == self.Lz and self.xy == self.xz == self.yz == 0)

    # -- lattice ------------------------------------------------------------------
    def get_box_vector(self, i):
        """Lattice vector i (Box.h:503-518)."""
        if i == 0:
            return np.array([self._L[0], 0, 0], dtype=np.float64)
        if i == 1:
            return np.array([self._L[1] * self._xy, self._L[1], 0], dtype=np.float64)
        if i == 2 and not self.is2D:
            return np.array([self._L[2] * self._xz, self._L[2] * self._yz, self._L[2]], dtype=np.float64)
        raise IndexError("Box lattice vector index requested does not exist.")

    @property
    def v1(self):
        return self.get_box_vector(0)

    @property
    def v2(self):
        return self.get_box_vector(1)

    @property
    def v3(self):
        return self.get_box_vector(2)

    def nearest_plane_distance(self):
        """Box.h:489-497, float32."""
        xy, xz, yz = self._xy, self._xz, self._yz
        t = xy * yz - xz
        d0 = self._L[0] / np.sqrt(_f32(1.0) + xy * xy + t * t)
        d1 = self._L[1] / np.sqrt(_f32(1.0) + yz * yz)
        return np.array([d0, d1, self._L[2]], dtype=_f32)

    # -- coordinate transforms (float32, reference operation order) -----------------
    def _frac(self, v):
        v = np.asarray(v, dtype=_f32)
        d = v - self._lo
        t2 = self._xz - self._yz * self._xy
        dx = d[..., 0] - (t2 * v[..., 2] + self._xy * v[..., 1])
        dy = d[..., 1] - self._yz * v[..., 2]
        with np.errstate(divide="ignore", invalid="ignore"):
            fx = dx / self._L[0]
            fy = dy / self._L[1]
            fz = d[..., 2] / self._L[2] if not self.is2D else np.zeros_like(dx)
        return np.stack([fx, fy, fz], axis=-1).astype(_f32)

    def _abs(self, f):
        f = np.asarray(f, dtype=_f32)
        v = self._lo + f * self._L
        x = v[..., 0] + (self._xy * v[..., 1] + self._xz * v[..., 2])
        y = v[..., 1] + self._yz * v[..., 2]
        z = v[..., 2] if not self.is2D else np.zeros_like(x)
        return np.stack([x, y, z], axis=-1).astype(_f32)

    def make_absolute(self, fractional_coordinates, out=None):
        f = np.asarray(fractional_coordinates, dtype=_f32)
        res = self._abs(np.atleast_2d(f)).reshape(f.shape)
        if out is not None:
            out[...] = res
            return out
        return res

    def make_fractional(self, absolute_coordinates, out=None):
        v = np.asarray(absolute_coordinates, dtype=_f32)
        res = self._frac(np.atleast_2d(v)).reshape(v.shape)
        if out is not None:
            out[...] = res
            return out
        return res

    def get_images(self, vecs):
        vecs = np.asarray(vecs, dtype=_f32)
        f = self._frac(np.atleast_2d(vecs)) - _f32(0.5)
        if self.is2D:
            f[..., 2] = 0
        img = np.where(f >= 0, f + _f32(0.5), f - _f32(0.5)).astype(np.int32)
        return img.reshape(vecs.shape)

    def wrap(self, vecs, out=None):
        """Box::wrap (Box.h:307-329): fmod(fmod(f, 1) + 1, 1) per periodic axis."""
        vecs = np.asarray(vecs, dtype=_f32)
        v = np.atleast_2d(vecs)
        f = self._frac(v)
        for a in range(3):
            if self._periodic[a]:
                f[..., a] = np.fmod(np.fmod(f[..., a], _f32(1.0)) + _f32(1.0), _f32(1.0))
        res = self._abs(f).reshape(vecs.shape)
        if out is not None:
            out[...] = res
            return out
        return res

    def unwrap(self, vecs, imgs, out=None):
        vecs = np.asarray(vecs, dtype=_f32)
        imgs = np.asarray(imgs)
        res = (vecs + self.get_box_vector(0).astype(_f32) * imgs[..., 0:1].astype(_f32)
               + self.get_box_vector(1).astype(_f32) * imgs[..., 1:2].astype(_f32))
        if not self.is2D:
            res = res + self.get_box_vector(2).astype(_f32) * imgs[..., 2:3].astype(_f32)
        res = res.astype(_f32)
        if out is not None:
            out[...] = res
            return out
        return res

    def compute_distances(self, query_points, points):
        q = np.atleast_2d(np.asarray(query_points, dtype=_f32))
        p = np.atleast_2d(np.asarray(points, dtype=_f32))
        if len(q) != len(p):
            raise ValueError("The number of query points and points must match.")
        r = self.wrap(p - q)
        return np.sqrt((r[:, 0] * r[:, 0] + r[:, 1] * r[:, 1]) + r[:, 2] * r[:, 2])

    def compute_all_distances(self, query_points, points):
        q = np.atleast_2d(np.asarray(query_points, dtype=_f32))
        p = np.atleast_2d(np.asarray(points, dtype=_f32))
        r = self.wrap((p[np.newaxis, :, :] - q[:, np.newaxis, :]).reshape(-1, 3))
        d = np.sqrt((r[:, 0] * r[:, 0] + r[:, 1] * r[:, 1]) + r[:, 2] * r[:, 2])
        return d.reshape(len(q), len(p))

    def contains(self, points):
        return np.all(self.get_images(np.atleast_2d(points)) == 0, axis=-1)

    # -- conversion -----------------------------------------------------------------
    def to_dict(self):
        return {"Lx": self.Lx, "Ly": self.Ly, "Lz": self.Lz, "xy": self.xy, "xz": self.xz, "yz": self.yz,
                "dimensions": self.dimensions}

    def to_matrix(self):
        return np.asarray([[self.Lx, self.xy * self.Ly, self.xz * self.Lz],
                           [0, self.Ly, self.yz * self.Lz],
                           [0, 0, self.Lz]])

    def to_box_lengths_and_angles(self):
        alpha = np.arccos((self.xy * self.xz + self.yz) / (np.sqrt(1 + self.xy**2) * np.sqrt(1 + self.xz**2 + self.yz**2)))
        beta = np.arccos(self.xz / np.sqrt(1 + self.xz**2 + self.yz**2))
        gamma = np.arccos(self.xy / np.sqrt(1 + self.xy**2))
        L1 = self.Lx
        a2 = [self.Ly * self.xy, self.Ly, 0]
        a3 = [self.Lz * self.xz, self.Lz * self.yz, self.Lz]
        return (L1, np.linalg.norm(a2), np.linalg.norm(a3), alpha, beta, gamma)

    def _c_box(self):
        from . import _lib

        b = _lib.fg_box()
        b.Lx, b.Ly, b.Lz = float(self._L[0]), float(self._L[1]), float(self._L[2])
        b.xy, b.xz, b.yz = float(self._xy), float(self._xz), float(self._yz)
        b.is2D = int(self.is2D)
        b.periodic_x, b.periodic_y, b.periodic_z = (int(p) for p in self._periodic)
        return b

    def _box7(self):
        return np.array([self.Lx, self.Ly, self.Lz, self.xy, self.xz, self.yz, 1.0 if self.is2D else 0.0], _f32)

    def __eq__(self, other):
        if not isinstance(other, Box):
            return False
        return (np.array_equal(self._L, other._L) and self._xy == other._xy and self._xz == other._xz
                and self._yz == other._yz and self.is2D == other.is2D and self._periodic == other._periodic)

    def __hash__(self):
        return hash((tuple(self._L.tolist()), float(self._xy), float(self._xz), float(self._yz), self.is2D))

    def __repr__(self):
        return ("freud.box.{cls}(Lx={Lx}, Ly={Ly}, Lz={Lz}, xy={xy}, xz={xz}, yz={yz}, is2D={is2D})").format(
            cls=type(self).__name__, Lx=self.Lx, Ly=self.Ly, Lz=self.Lz, xy=self.xy, xz=self.xz, yz=self.yz,
            is2D=self.is2D)

    def __str__(self):
        return repr(self)

    def __mul__(self, scale):
        if scale > 0:
            return self.__class__(Lx=self.Lx * scale, Ly=self.Ly * scale, Lz=self.Lz * scale, xy=self.xy,
                                  xz=self.xz, yz=self.yz, is2D=self.is2D)
        raise ValueError("Box can only be multiplied by positive values.")

    def __rmul__(self, scale):
        return self * scale
