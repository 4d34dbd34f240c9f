"""Radial distribution function and pair correlation function, API-compatible
with freud.density.RDF (freud/density.py:535-696) and
freud.density.CorrelationFunction (freud/density.py:28-177). Pair finding and
binning run on the GPU; RDF bin counts are exact uint64 on the device and
reported as the reference's uint32, and rdf / n_r use the reference's float32
normalisation (RDF.cc:73-99)."""

import ctypes

import numpy as np

from . import _lib
from .box import Box
from .locality import FrameBatch, NeighborList, _QueryArgs, _SpatialHistogram1D
from .util import _Compute, _convert_array


class RDF(_SpatialHistogram1D):
    """Computes g(r) and the cumulative N(r).

    Args:
        bins (unsigned int): number of bins.
        r_max (float): largest distance binned.
        r_min (float, optional): smallest distance binned (default 0).
        normalization_mode (str, optional): ``'exact'`` or ``'finite_size'``.
    """

    def __init__(self, bins, r_max, r_min=0, normalization_mode="exact"):
        h = ctypes.c_void_p()
        _lib.check(_lib.lib.fg_rdf_create(int(bins), float(r_max), float(r_min), ctypes.byref(h)))
        self._handle = _lib.Handle(h, _lib.lib.fg_rdf_destroy)
        self._bins = int(bins)
        self.mode = normalization_mode
        self.r_max = r_max
        self._r_min = r_min

    @property
    def _h(self):
        return self._handle.value

    @property
    def mode(self):
        return self._mode

    @mode.setter
    def mode(self, value):
        if value not in ("exact", "finite_size"):
            raise ValueError("An invalid normalization mode was provided.")
        self._mode = value
        _lib.check(_lib.lib.fg_rdf_set_mode(self._h, int(value == "finite_size")))

    def _reset(self):
        _lib.check(_lib.lib.fg_rdf_reset(self._h))

    def compute(self, system, query_points=None, neighbors=None, reset=True):
        """Accumulate the pair distances of one frame (reset=False keeps adding frames)."""
        if reset:
            self._reset()
        if isinstance(system, FrameBatch):
            # every frame in one pass: same counts as one compute(reset=False) per frame
            if query_points is not None or isinstance(neighbors, NeighborList):
                raise ValueError("a FrameBatch is queried against itself; query_points and NeighborList "
                                 "neighbors are not supported")
            query_args = self.default_query_args if neighbors is None else dict(neighbors)
            query_args.setdefault("exclude_ii", True)
            qargs = _QueryArgs.from_dict(query_args)
            _lib.check(_lib.lib.fg_rdf_accumulate_frames(self._h, system._h, ctypes.byref(qargs._c())))
            return self
        nq, nlist, qargs, l_query_points, num_query_points = self._preprocess_arguments(
            system, query_points, neighbors)
        qp_arg = nq._query_points_arg(l_query_points)
        _lib.check(_lib.lib.fg_rdf_accumulate(
            self._h, nq._h, _lib.ptr(qp_arg), num_query_points, None if nlist is None else nlist._h,
            ctypes.byref(qargs._c())))
        return self

    def _get(self):
        c = np.zeros(self._bins, np.uint32)
        g = np.zeros(self._bins, np.float32)
        nr = np.zeros(self._bins, np.float32)
        _lib.check(_lib.lib.fg_rdf_get(self._h, _lib.ptr(c), _lib.ptr(g), _lib.ptr(nr)))
        return c, g, nr

    @_Compute._computed_property
    def rdf(self):
        return self._get()[1]

    @_Compute._computed_property
    def n_r(self):
        return self._get()[2]

    @_Compute._computed_property
    def bin_counts(self):
        return self._get()[0]

    @_Compute._computed_property
    def bin_counts_u64(self):
        """Full-width uint64 bin counts (the reference stores uint32)."""
        c = np.zeros(self._bins, np.uint64)
        _lib.check(_lib.lib.fg_rdf_get_u64(self._h, _lib.ptr(c), None, None))
        return c

    @_Compute._computed_property
    def rdf_fp64(self):
        """g(r) normalised in FP64 from the uint64 counts."""
        g = np.zeros(self._bins, np.float64)
        _lib.check(_lib.lib.fg_rdf_get_u64(self._h, None, _lib.ptr(g), None))
        return g

    @_Compute._computed_property
    def n_r_fp64(self):
        nr = np.zeros(self._bins, np.float64)
        _lib.check(_lib.lib.fg_rdf_get_u64(self._h, None, None, _lib.ptr(nr)))
        return nr

    @_Compute._computed_property
    def box(self):
        b = _lib.fg_box()
        _lib.check(_lib.lib.fg_rdf_state(self._h, ctypes.byref(b), None, None, None))
        return Box(b.Lx, b.Ly, b.Lz, b.xy, b.xz, b.yz, bool(b.is2D))

    @property
    def bin_edges(self):
        e = np.zeros(self._bins + 1, np.float32)
        _lib.check(_lib.lib.fg_rdf_bin_edges(self._h, _lib.ptr(e), None))
        return e.astype(np.float64)

    @property
    def bin_centers(self):
        c = np.zeros(self._bins, np.float32)
        _lib.check(_lib.lib.fg_rdf_bin_edges(self._h, None, _lib.ptr(c)))
        return c.astype(np.float64)

    @property
    def bounds(self):
        return (float(np.float32(self._r_min)), float(np.float32(self.r_max)))

    @property
    def nbins(self):
        return self._bins

    def __repr__(self):
        return "freud.density.{}(bins={}, r_max={}, r_min={})".format(
            type(self).__name__, self._bins, self.bounds[1], self.bounds[0])


class CorrelationFunction(_SpatialHistogram1D):
    """Complex pairwise correlation function C(r) = <s1*(0) s2(r)>
    (freud/density.py:28-177, CorrelationFunction.cc:26-99): the average of
    conj(values[j]) * query_values[i] over the bonds (i, j) whose distance falls in
    each bin. Bonds are found on the GPU and the products summed in FP64 there.

    Args:
        bins (unsigned int): number of bins.
        r_max (float): largest distance binned.
    """

    def __init__(self, bins, r_max):
        h = ctypes.c_void_p()
        _lib.check(_lib.lib.fg_cf_create(int(bins), float(r_max), ctypes.byref(h)))
        self._handle = _lib.Handle(h, _lib.lib.fg_cf_destroy)
        self._bins = int(bins)
        self.r_max = r_max
        self.is_complex = False

    @property
    def _h(self):
        return self._handle.value

    def _reset(self):
        _lib.check(_lib.lib.fg_cf_reset(self._h))

    def compute(self, system, values, query_points=None, query_values=None, neighbors=None, reset=True):
        """Accumulate the correlation of one frame (reset=False keeps adding frames)."""
        if reset:
            self.is_complex = False
            self._reset()
        nq, nlist, qargs, l_query_points, num_query_points = self._preprocess_arguments(
            system, query_points, neighbors)
        self.is_complex = (self.is_complex or bool(np.any(np.iscomplex(values)))
                           or bool(np.any(np.iscomplex(query_values))))
        values = _convert_array(values, shape=(nq._n_points,), dtype=np.complex128)
        if query_values is None:
            query_values = values
        else:
            query_values = _convert_array(query_values, shape=(num_query_points,), dtype=np.complex128)
        qp_arg = nq._query_points_arg(l_query_points)
        qv_arg = None if query_values is values else query_values
        _lib.check(_lib.lib.fg_cf_accumulate(
            self._h, nq._h, _lib.ptr(values), len(values), _lib.ptr(qp_arg), num_query_points, _lib.ptr(qv_arg),
            len(query_values), None if nlist is None else nlist._h, ctypes.byref(qargs._c())))
        return self

    @_Compute._computed_property
    def correlation(self):
        """Average product per bin (complex when any value was complex)."""
        out = np.zeros(self._bins, np.complex128)
        _lib.check(_lib.lib.fg_cf_get(self._h, None, _lib.ptr(out)))
        return out if self.is_complex else np.real(out)

    @_Compute._computed_property
    def bin_counts(self):
        c = np.zeros(self._bins, np.uint32)
        _lib.check(_lib.lib.fg_cf_get(self._h, _lib.ptr(c), None))
        return c

    @_Compute._computed_property
    def box(self):
        b = _lib.fg_box()
        _lib.check(_lib.lib.fg_cf_state(self._h, ctypes.byref(b), None))
        return Box(b.Lx, b.Ly, b.Lz, b.xy, b.xz, b.yz, bool(b.is2D))

    @property
    def bin_edges(self):
        e = np.zeros(self._bins + 1, np.float32)
        _lib.check(_lib.lib.fg_cf_bin_edges(self._h, _lib.ptr(e), None))
        return e.astype(np.float64)

    @property
    def bin_centers(self):
        c = np.zeros(self._bins, np.float32)
        _lib.check(_lib.lib.fg_cf_bin_edges(self._h, None, _lib.ptr(c)))
        return c.astype(np.float64)

    @property
    def bounds(self):
        return (0.0, float(np.float32(self.r_max)))

    @property
    def nbins(self):
        return self._bins

    @property
    def bins(self):
        return self._bins

    def __repr__(self):
        return "freud.density.{}(bins={}, r_max={})".format(type(self).__name__, self._bins, self.r_max)
