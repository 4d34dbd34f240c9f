"""Potentials of mean force and torque, API-compatible with freud.pmft
(freud/pmft.py:58-589; PMFTR12.cc, PMFTXYT.cc, PMFTXY.cc, PMFTXYZ.cc). Bonds are
found and binned on the GPU; bin counts are exact integers and the pair
correlation function uses the reference's float32 normalisation (PMFT.h:70-82)."""

import ctypes

import numpy as np

from . import _lib
from .box import Box
from .locality import _SpatialHistogram
from .util import _Compute, _convert_array

_R12, _XYT, _XY, _XYZ = 0, 1, 2, 3


def _quat_to_z_angle(orientations, num_points):
    """Angles of z-axis rotation quaternions (freud/pmft.py:58-81): a 1D array of
    length 4 (unless there are exactly 4 points) or an (N, 4) array is read as
    quaternions (w, x, y, z) and converted with the axis-angle relation angle =
    2 arccos(w), axis = v / sin(angle / 2) of the normalised quaternion; any
    other array is already angles."""
    is_quat = (orientations.ndim == 1 and orientations.shape[0] == 4 and num_points != 4) or (
        orientations.ndim == 2 and orientations.shape[1] == 4)
    if not is_quat:
        return orientations
    q = np.atleast_2d(np.asarray(orientations, dtype=np.float64))
    q = q / np.linalg.norm(q, axis=-1, keepdims=True)
    angles = 2.0 * np.arccos(np.clip(q[:, 0], -1.0, 1.0))
    half = np.sin(angles / 2.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        axes = np.where(half[:, None] != 0, q[:, 1:] / half[:, None], np.array([1.0, 0.0, 0.0]))
    if not (np.allclose(angles, 0) or np.allclose(axes, [0, 0, 1])):
        raise ValueError("Orientations provided as quaternions must represent rotations about the z-axis.")
    return angles.reshape(orientations.shape[:-1])


def _gen_angle_array(orientations, shape):
    """float32 angles of the given shape (freud/pmft.py:84-94)."""
    return _convert_array(np.atleast_1d(_quat_to_z_angle(np.asarray(orientations).squeeze(), shape[0])),
                          shape=shape)


class _PMFT(_SpatialHistogram):
    """Common part of the PMFT classes (freud/pmft.py:97-121)."""

    def _create(self, kind, maxes, bins):
        self._kind = kind
        h = ctypes.c_void_p()
        m = np.ascontiguousarray(maxes, dtype=np.float32)
        b = np.ascontiguousarray(bins, dtype=np.uint32)
        _lib.check(_lib.lib.fg_pmft_create(kind, _lib.ptr(m), _lib.ptr(b), ctypes.byref(h)))
        self._handle = _lib.Handle(h, _lib.lib.fg_pmft_destroy)
        self._shape = tuple(int(x) for x in bins)

    @property
    def _h(self):
        return self._handle.value

    def _reset(self):
        _lib.check(_lib.lib.fg_pmft_reset(self._h))

    def _accumulate(self, nq, orientations, query_points, num_query_points, query_orientations, equiv, nlist,
                    qargs):
        qp_arg = nq._query_points_arg(query_points)
        n_or = 0 if orientations is None else len(orientations)
        n_qo = 0 if query_orientations is None else len(query_orientations)
        n_eq = 0 if equiv is None else len(equiv)
        _lib.check(_lib.lib.fg_pmft_accumulate(
            self._h, nq._h, _lib.ptr(orientations), n_or, _lib.ptr(qp_arg), num_query_points,
            _lib.ptr(query_orientations), n_qo, _lib.ptr(equiv), n_eq, None if nlist is None else nlist._h,
            ctypes.byref(qargs._c())))

    def _axis(self, a):
        n = ctypes.c_uint32()
        _lib.check(_lib.lib.fg_pmft_axis(self._h, a, None, None, None, ctypes.byref(n)))
        e = np.zeros(n.value + 1, np.float32)
        c = np.zeros(n.value, np.float32)
        bnd = np.zeros(2, np.float32)
        _lib.check(_lib.lib.fg_pmft_axis(self._h, a, _lib.ptr(e), _lib.ptr(c), _lib.ptr(bnd), None))
        return e, c, bnd

    def _get(self):
        n = int(np.prod(self._shape))
        c = np.zeros(n, np.uint32)
        g = np.zeros(n, np.float32)
        _lib.check(_lib.lib.fg_pmft_get(self._h, _lib.ptr(c), _lib.ptr(g)))
        return c.reshape(self._shape), g.reshape(self._shape)

    @_Compute._computed_property
    def bin_counts(self):
        return self._get()[0]

    @_Compute._computed_property
    def _pcf(self):
        return self._get()[1]

    @_Compute._computed_property
    def pmft(self):
        """The discrete potential of mean force and torque, -log(pcf)."""
        with np.errstate(divide="ignore"):
            return -np.log(np.copy(self._pcf))

    @_Compute._computed_property
    def box(self):
        b = _lib.fg_box()
        _lib.check(_lib.lib.fg_pmft_state(self._h, ctypes.byref(b), None))
        return Box(b.Lx, b.Ly, b.Lz, b.xy, b.xz, b.yz, bool(b.is2D))

    @property
    def bin_centers(self):
        return [self._axis(a)[1].astype(np.float64) for a in range(len(self._shape))]

    @property
    def bin_edges(self):
        return [self._axis(a)[0].astype(np.float64) for a in range(len(self._shape))]

    @property
    def bounds(self):
        return [tuple(float(x) for x in self._axis(a)[2]) for a in range(len(self._shape))]

    @property
    def nbins(self):
        return list(self._shape)


class PMFTR12(_PMFT):
    """PMFT in (r, theta1, theta2) for 2D systems (freud/pmft.py:124-221).

    Args:
        r_max (float): largest distance binned.
        bins (unsigned int or sequence of 3): bins in r, theta1, theta2.
    """

    def __init__(self, r_max, bins):
        try:
            n_r, n_t1, n_t2 = bins
        except TypeError:
            n_r = n_t1 = n_t2 = bins
        self._create(_R12, [r_max], [n_r, n_t1, n_t2])
        self.r_max = r_max

    def compute(self, system, orientations, query_points=None, query_orientations=None, neighbors=None, reset=True):
        if reset:
            self._reset()
        nq, nlist, qargs, query_points, num_query_points = self._preprocess_arguments(system, query_points, neighbors)
        orientations = _gen_angle_array(orientations, shape=(nq._n_points,))
        if query_orientations is None:
            query_orientations = orientations
        else:
            query_orientations = _gen_angle_array(query_orientations, shape=(num_query_points,))
        self._accumulate(nq, orientations, query_points, num_query_points, query_orientations, None, nlist, qargs)
        return self

    def __repr__(self):
        return "freud.pmft.{cls}(r_max={r_max}, bins=({bins}))".format(
            cls=type(self).__name__, r_max=self.r_max, bins=", ".join(str(b) for b in self.nbins))


class PMFTXYT(_PMFT):
    """PMFT in (x, y, theta) for 2D systems (freud/pmft.py:224-325).

    Args:
        x_max (float), y_max (float): half-widths of the binned region.
        bins (unsigned int or sequence of 3): bins in x, y, theta.
    """

    def __init__(self, x_max, y_max, bins):
        try:
            n_x, n_y, n_t = bins
        except TypeError:
            n_x = n_y = n_t = bins
        self._create(_XYT, [x_max, y_max], [n_x, n_y, n_t])
        self.r_max = np.sqrt(x_max ** 2 + y_max ** 2)

    def compute(self, system, orientations, query_points=None, query_orientations=None, neighbors=None, reset=True):
        if reset:
            self._reset()
        nq, nlist, qargs, query_points, num_query_points = self._preprocess_arguments(system, query_points, neighbors)
        orientations = _gen_angle_array(orientations, shape=(nq._n_points,))
        if query_orientations is None:
            query_orientations = orientations
        else:
            query_orientations = _gen_angle_array(query_orientations, shape=(num_query_points,))
        self._accumulate(nq, orientations, query_points, num_query_points, query_orientations, None, nlist, qargs)
        return self

    def __repr__(self):
        bounds = self.bounds
        return "freud.pmft.{cls}(x_max={x_max}, y_max={y_max}, bins=({bins}))".format(
            cls=type(self).__name__, x_max=bounds[0][1], y_max=bounds[1][1],
            bins=", ".join(str(b) for b in self.nbins))


class PMFTXY(_PMFT):
    """PMFT in (x, y) for 2D systems (freud/pmft.py:328-453).

    Args:
        x_max (float), y_max (float): half-widths of the binned region.
        bins (unsigned int or sequence of 2): bins in x, y.
    """

    def __init__(self, x_max, y_max, bins):
        try:
            n_x, n_y = bins
        except TypeError:
            n_x = n_y = bins
        self._create(_XY, [x_max, y_max], [n_x, n_y])
        self.r_max = np.sqrt(x_max ** 2 + y_max ** 2)

    def compute(self, system, query_orientations, query_points=None, neighbors=None, reset=True):
        if reset:
            self._reset()
        nq, nlist, qargs, query_points, num_query_points = self._preprocess_arguments(system, query_points, neighbors)
        query_orientations = _gen_angle_array(query_orientations, shape=(num_query_points,))
        self._accumulate(nq, None, query_points, num_query_points, query_orientations, None, nlist, qargs)
        return self

    @_Compute._computed_property
    def bin_counts(self):
        return np.squeeze(self._get()[0])

    def __repr__(self):
        bounds = self.bounds
        return "freud.pmft.{cls}(x_max={x_max}, y_max={y_max}, bins=({bins}))".format(
            cls=type(self).__name__, x_max=bounds[0][1], y_max=bounds[1][1],
            bins=", ".join(str(b) for b in self.nbins))


class PMFTXYZ(_PMFT):
    """PMFT in (x, y, z) for 3D systems (freud/pmft.py:456-589).

    Args:
        x_max (float), y_max (float), z_max (float): half-widths of the binned region.
        bins (unsigned int or sequence of 3): bins in x, y, z.
        shiftvec (list): vector from the origin to the centre of the PMFT.
    """

    def __init__(self, x_max, y_max, z_max, bins, shiftvec=None):
        if shiftvec is None:
            shiftvec = [0, 0, 0]
        try:
            n_x, n_y, n_z = bins
        except TypeError:
            n_x = n_y = n_z = bins
        self._create(_XYZ, [x_max, y_max, z_max], [n_x, n_y, n_z])
        self.shiftvec = np.array(shiftvec, dtype=np.float32)
        self.r_max = np.sqrt(x_max ** 2 + y_max ** 2 + z_max ** 2)

    def compute(self, system, query_orientations, query_points=None, equiv_orientations=None, neighbors=None,
                reset=True):
        if reset:
            self._reset()
        nq, nlist, qargs, query_points, num_query_points = self._preprocess_arguments(system, query_points, neighbors)
        if query_points is not None or np.any(self.shiftvec != 0):
            # query_points - shiftvec (freud/pmft.py:553); a zero shift of the
            # system's own points leaves them as they are on the device
            if query_points is None:
                query_points = nq.points
            query_points = np.ascontiguousarray(query_points - self.shiftvec.reshape(1, 3), dtype=np.float32)
        query_orientations = _convert_array(np.atleast_1d(query_orientations), shape=(num_query_points, 4))
        if equiv_orientations is None:
            equiv_orientations = np.array([[1, 0, 0, 0]], dtype=np.float32)
        else:
            equiv_orientations = _convert_array(equiv_orientations, shape=(None, 4))
        self._accumulate(nq, None, query_points, num_query_points, query_orientations, equiv_orientations, nlist,
                         qargs)
        return self

    def __repr__(self):
        bounds = self.bounds
        return ("freud.pmft.{cls}(x_max={x_max}, y_max={y_max}, z_max={z_max}, bins=({bins}), "
                "shiftvec={shiftvec})").format(
            cls=type(self).__name__, x_max=bounds[0][1], y_max=bounds[1][1], z_max=bounds[2][1],
            bins=", ".join(str(b) for b in self.nbins), shiftvec=self.shiftvec.tolist())
