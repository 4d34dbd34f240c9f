"""Neighbour queries and neighbour lists, API-compatible with freud.locality
(freud/locality.py:39-1091). Queries run on the GPU through the C ABI in
include/freud_gb300.h; NeighborList arrays live on the device and are copied to
host numpy arrays (read-only, cached) on first access.
"""

import inspect

import numpy as np

from . import _lib
from .box import Box
from .util import _Compute, _convert_array, _convert_box

ITERATOR_TERMINATOR = None

NO_DEFAULT_QUERY_ARGS_MESSAGE = (
    "Query arguments must be provided for {} objects since there is no default set of arguments."
)


class _QueryArgs:
    """Query arguments (NeighborQuery.h:60-73; freud/locality.py:39-175)."""

    def __init__(self, mode=None, r_min=None, r_max=None, r_guess=None, num_neighbors=None, exclude_ii=None,
                 scale=None, **kwargs):
        self.mode = mode
        self._r_max = -1.0
        self._r_min = 0.0
        self._r_guess = -1.0
        self._num_neighbors = _lib.DEFAULT_NUM_NEIGHBORS
        self._exclude_ii = False
        self._scale = -1.0
        if r_max is not None:
            self.r_max = r_max
        if r_min is not None:
            self.r_min = r_min
        if r_guess is not None:
            self.r_guess = r_guess
        if num_neighbors is not None:
            self.num_neighbors = num_neighbors
        if exclude_ii is not None:
            self.exclude_ii = exclude_ii
        if scale is not None:
            self.scale = scale
        if len(kwargs) > 0:
            err_str = ", ".join("{} = {}".format(k, v) for k, v in kwargs.items())
            raise ValueError("The following invalid query arguments were provided: " + err_str)

    def update(self, qargs):
        if qargs is None:
            return
        for arg in qargs:
            if hasattr(self, arg):
                setattr(self, arg, qargs[arg])
            else:
                raise ValueError("An invalid query argument was provided.")

    @classmethod
    def from_dict(cls, mapping):
        return cls(**mapping)

    @property
    def mode(self):
        return self._mode

    @mode.setter
    def mode(self, value):
        if value == "none" or value is None:
            self._mode = None
        elif value in ("ball", "nearest"):
            self._mode = value
        else:
            raise ValueError("An invalid mode was provided.")

    def _f32(self, v):
        return float(np.float32(v))

    @property
    def r_guess(self):
        return self._r_guess

    @r_guess.setter
    def r_guess(self, value):
        self._r_guess = self._f32(value)

    @property
    def r_min(self):
        return self._r_min

    @r_min.setter
    def r_min(self, value):
        self._r_min = self._f32(value)

    @property
    def r_max(self):
        return self._r_max

    @r_max.setter
    def r_max(self, value):
        self._r_max = self._f32(value)

    @property
    def num_neighbors(self):
        return self._num_neighbors

    @num_neighbors.setter
    def num_neighbors(self, value):
        self._num_neighbors = int(value) & 0xFFFFFFFF

    @property
    def exclude_ii(self):
        return self._exclude_ii

    @exclude_ii.setter
    def exclude_ii(self, value):
        self._exclude_ii = bool(value)

    @property
    def scale(self):
        return self._scale

    @scale.setter
    def scale(self, value):
        self._scale = self._f32(value)

    def _c(self):
        mode = {None: _lib.MODE_NONE, "ball": _lib.MODE_BALL, "nearest": _lib.MODE_NEAREST}[self._mode]
        return _lib.make_args(mode, self._num_neighbors, self._r_max, self._r_min, self._r_guess, self._scale,
                              self._exclude_ii)

    def __repr__(self):
        return ("freud.locality.{}(mode={}, r_max={}, num_neighbors={}, exclude_ii={}, scale={})".format(
            type(self).__name__, self.mode, self.r_max, self.num_neighbors, self.exclude_ii, self.scale))

    def __str__(self):
        return repr(self)


def _match_class_path(obj, *matches):
    return any(c.__module__ + "." + c.__name__ in matches for c in inspect.getmro(type(obj)))


def _as_box_points(system):
    """(box, points) from a system-like object: a (box, points) sequence, a GSD
    frame (gsd.hoomd.Frame / Snapshot, hoomd Snapshot, freud_gb300.gsd.Frame:
    box from configuration.box, 2D frames with Lz, xz, yz zeroed, points from
    particles.position; freud/locality.py:327-336) or an object with box and
    points attributes."""
    if _match_class_path(system, "gsd.hoomd.Frame", "gsd.hoomd.Snapshot", "hoomd.snapshot.Snapshot",
                         "freud_gb300.gsd.Frame"):
        box = np.array(system.configuration.box)
        if system.configuration.dimensions == 2:
            box[[2, 4, 5]] = 0
        return box, system.particles.position
    if hasattr(system, "box") and hasattr(system, "points"):
        return system.box, system.points
    return system


class NeighborQueryResult:
    """Lazy result of NeighborQuery.query (freud/locality.py:178-229)."""

    def __init__(self, nq, points, query_args):
        self._nq = nq
        # query() has already converted the points; keep them without another copy
        self._points = np.ascontiguousarray(points, dtype=np.float32)
        self._query_args = query_args

    def __iter__(self):
        # nearest-neighbour iterators return each point's bonds by distance
        by_distance = self._nq._is_nearest(self._query_args)
        nlist = self.toNeighborList(sort_by_distance=by_distance)
        ij = nlist[:]
        d = nlist.distances
        for b in range(len(ij)):
            yield (int(ij[b, 0]), int(ij[b, 1]), float(d[b]))

    def toNeighborList(self, sort_by_distance=False):
        """Convert the query result to a NeighborList (reference order: by point
        index, or by distance when sort_by_distance)."""
        return self._nq._query_nlist(self._points, self._query_args, sort_by_distance)


class NeighborQuery:
    """A set of points in a box that can be queried for neighbours (abstract)."""

    def __init__(self):
        raise RuntimeError("The NeighborQuery class is abstract, and should not be directly instantiated")

    def _init(self, box, points, kind, cell_width=0.0):
        b = _convert_box(box)
        self._box = b
        pts = _convert_array(points, shape=(None, 3))
        self._kind = kind
        h = _lib.ctypes.c_void_p()
        _lib.check(_lib.lib.fg_nq_create(_lib.ctypes.byref(b._c_box()), _lib.ptr(pts), len(pts), kind,
                                         float(cell_width), _lib.ctypes.byref(h)))
        self._handle = _lib.Handle(h, _lib.lib.fg_nq_destroy)
        # the library keeps its own copy of the points (on the device); the host
        # copy behind .points is made from it on first use
        self._n_points = len(pts)
        self._points = None

    @property
    def _h(self):
        return self._handle.value

    @classmethod
    def from_system(cls, system, dimensions=None):
        """Create a NeighborQuery from a system-like object: a NeighborQuery, a
        (box, points) sequence, or an object with box and points attributes."""

        if isinstance(system, cls):
            return system
        system = _as_box_points(system)
        if cls == NeighborQuery:
            return _RawPoints(*system)
        return cls(*system)

    @property
    def box(self):
        return self._box

    @property
    def points(self):
        if self._points is None:
            pts = np.empty((self._n_points, 3), np.float32)
            _lib.check(_lib.lib.fg_nq_get_points(self._h, _lib.ptr(pts)))
            self._points = pts
        return self._points

    def query(self, query_points, query_args):
        query_points = _convert_array(np.atleast_2d(query_points), shape=(None, 3))
        args = _QueryArgs.from_dict(query_args)
        return NeighborQueryResult(self, query_points, args)

    # -- internals ------------------------------------------------------------------
    def _query_points_arg(self, query_points):
        """query_points as passed to the library: None for this object's own host
        copy (already on the device); anything else is uploaded, and the library
        compares it with the object's points on the device and reuses the
        object's cell grid when they are equal."""
        if query_points is None or query_points is self._points:
            return None
        return np.ascontiguousarray(query_points, dtype=np.float32)

    def _is_nearest(self, qargs):
        return qargs.mode == "nearest" or (qargs.mode is None and qargs.num_neighbors != _lib.DEFAULT_NUM_NEIGHBORS)

    def _query_nlist(self, query_points, qargs, sort_by_distance=False):
        query_points = np.ascontiguousarray(query_points, dtype=np.float32)
        qp = self._query_points_arg(query_points)
        h = _lib.ctypes.c_void_p()
        _lib.check(_lib.lib.fg_nq_query(self._h, _lib.ptr(qp), len(query_points), _lib.ctypes.byref(qargs._c()),
                                        int(bool(sort_by_distance)), _lib.ctypes.byref(h)))
        return NeighborList._from_handle(h)


class _RawPoints(NeighborQuery):
    """(box, points) with no user-built structure; queried with AABB arithmetic
    (freud/locality/RawPoints.h:30-77)."""

    def __init__(self, box, points):
        self._init(box, points, _lib.NQ_RAWPOINTS)


class AABBQuery(NeighborQuery):
    """Neighbour queries with freud's AABBQuery arithmetic (r = p_j - (q + image))."""

    def __init__(self, box, points):
        self._init(box, points, _lib.NQ_AABB)


class LinkCell(NeighborQuery):
    """Neighbour queries with freud's LinkCell arithmetic (r = box.wrap(p_j - q))."""

    def __init__(self, box, points, cell_width=0):
        self._init(box, points, _lib.NQ_LINKCELL, cell_width)

    @property
    def cell_width(self):
        out = _lib.ctypes.c_float()
        _lib.check(_lib.lib.fg_nq_cell_width(self._h, _lib.ctypes.byref(out)))
        return out.value


class CellQuery(NeighborQuery):
    """Neighbour queries with freud's CellQuery arithmetic (freud/locality.py:900-921):
    the points plus ghost copies of those within r_max of a box face, on a padded
    axis-aligned grid of r_max cells; r = g_j - q (CellIterator.h:173). Ball
    queries (r_max) only."""

    def __init__(self, box, points):
        self._init(box, points, _lib.NQ_CELLQUERY)


class FrameBatch:
    """Many (box, points) systems of uneven N held on the GPU together, so a
    compute runs over every frame in one launch per stage instead of one
    pipeline per frame. ``RDF.compute(batch, reset=False)`` equals calling
    ``RDF.compute((box, points), reset=False)`` frame by frame, and
    ``Steinhardt.compute(batch, neighbors)`` computes every frame with its own
    neighbours (per-particle outputs concatenated in frame order, ``order`` per
    frame). Frames use AABB pair arithmetic, as (box, points) systems do.

    Args:
        frames: iterable of (box, points) systems (or objects with ``box`` and
            ``points``), each with at least one point.
    """

    def __init__(self, frames):
        boxes, pts = [], []
        for system in frames:
            box, points = _as_box_points(system)
            b = _convert_box(box)
            boxes.append(b._c_box())
            pts.append(_convert_array(points, shape=(None, 3)))
        self._init(boxes, pts)

    def _init(self, boxes, pts):
        if len(boxes) == 0:
            raise ValueError("a FrameBatch needs at least one frame")
        self._offsets = np.zeros(len(boxes) + 1, dtype=np.uint64)
        self._offsets[1:] = np.cumsum([len(p) for p in pts])
        self._boxes = (_lib.fg_box * len(boxes))(*boxes)
        # each frame's float32 array goes to its slice of the device buffer (no
        # host-side concatenation)
        self._host_total = int(self._offsets[-1])
        ptrs = (_lib.ctypes.c_void_p * len(pts))(*[p.ctypes.data for p in pts])
        h = _lib.ctypes.c_void_p()
        _lib.check(_lib.lib.fg_frames_create_list(self._boxes, ptrs, _lib.ptr(self._offsets), len(boxes),
                                                  _lib.ctypes.byref(h)))
        self._handle = _lib.Handle(h, _lib.lib.fg_frames_destroy)

    @classmethod
    def from_device(cls, boxes, device_points_ptr, frame_offsets, keepalive=None):
        """A batch over points already on the GPU: ``device_points_ptr`` is the
        address of a contiguous (total, 3) float32 device array (e.g.
        ``tensor.data_ptr()``), ``frame_offsets`` the F + 1 ascending point
        offsets. ``keepalive`` (e.g. the tensor) is held by the batch."""
        self = cls.__new__(cls)
        c_boxes = [_convert_box(b)._c_box() for b in boxes]
        offs = np.asarray(frame_offsets, dtype=np.uint64)
        if len(offs) != len(c_boxes) + 1:
            raise ValueError("frame_offsets needs one more entry than boxes")
        if len(c_boxes) == 0:
            raise ValueError("a FrameBatch needs at least one frame")
        self._offsets = np.ascontiguousarray(offs)
        self._boxes = (_lib.fg_box * len(c_boxes))(*c_boxes)
        self._host_total = None
        self._keepalive = keepalive
        h = _lib.ctypes.c_void_p()
        _lib.check(_lib.lib.fg_frames_create_device(self._boxes, _lib.ctypes.c_void_p(device_points_ptr),
                                                    _lib.ptr(self._offsets), len(c_boxes), _lib.ctypes.byref(h)))
        self._handle = _lib.Handle(h, _lib.lib.fg_frames_destroy)
        return self

    @property
    def _h(self):
        return self._handle.value

    @property
    def num_frames(self):
        return len(self._offsets) - 1

    @property
    def frame_offsets(self):
        return self._offsets.copy()

    @property
    def num_points(self):
        """Points per frame."""
        return np.diff(self._offsets).astype(np.int64)

    def box(self, f):
        b = self._boxes[f]
        return Box(b.Lx, b.Ly, b.Lz, b.xy, b.xz, b.yz, bool(b.is2D))

    def set_points(self, points):
        """New positions (same frames and N, all frames concatenated) for a batch
        built from host points."""
        pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        if self._host_total is None or len(pts) != self._host_total:
            raise ValueError("set_points needs the same total number of points as the batch")
        _lib.check(_lib.lib.fg_frames_set_points(self._h, _lib.ptr(pts)))


class NeighborList:
    """Bonds between query points and points, sorted by query point index
    (freud/locality.py:443-751). Arrays are device-resident; properties return
    read-only host copies."""

    def __init__(self, _null=False):
        self._handle = None
        self._cache = {}
        if not _null:
            h = _lib.ctypes.c_void_p()
            empty = np.zeros(0, np.uint32)
            _lib.check(_lib.lib.fg_nlist_from_arrays(0, _lib.ptr(empty), 0, _lib.ptr(empty), 0, None, None,
                                                     _lib.ctypes.byref(h)))
            self._handle = _lib.Handle(h, _lib.lib.fg_nlist_destroy)

    @classmethod
    def _from_handle(cls, h):
        nl = cls(_null=True)
        nl._handle = _lib.Handle(h, _lib.lib.fg_nlist_destroy)
        return nl

    @property
    def _h(self):
        return None if self._handle is None else self._handle.value

    @classmethod
    def from_arrays(cls, num_query_points, num_points, query_point_indices, point_indices, vectors, weights=None):
        query_point_indices = _convert_array(query_point_indices, shape=(None,), dtype=np.uint32).copy()
        point_indices = _convert_array(point_indices, shape=query_point_indices.shape, dtype=np.uint32).copy()
        vectors = _convert_array(vectors, shape=(len(query_point_indices), 3), dtype=np.float32).copy()
        if weights is None:
            weights = np.ones(query_point_indices.shape, dtype=np.float32)
        weights = _convert_array(weights, shape=query_point_indices.shape).copy()
        h = _lib.ctypes.c_void_p()
        _lib.check(_lib.lib.fg_nlist_from_arrays(len(query_point_indices), _lib.ptr(query_point_indices),
                                                 int(num_query_points), _lib.ptr(point_indices), int(num_points),
                                                 _lib.ptr(vectors), _lib.ptr(weights), _lib.ctypes.byref(h)))
        return cls._from_handle(h)

    @classmethod
    def all_pairs(cls, system, query_points=None, exclude_ii=True):
        nq = NeighborQuery.from_system(system)
        points = nq.points
        if query_points is None:
            query_points = points
        points = _convert_array(points, shape=points.shape, dtype=np.float32)
        query_points = _convert_array(np.atleast_2d(query_points), shape=(None, 3), dtype=np.float32)
        h = _lib.ctypes.c_void_p()
        _lib.check(_lib.lib.fg_nlist_all_pairs(_lib.ctypes.byref(nq.box._c_box()), _lib.ptr(points), len(points),
                                               _lib.ptr(query_points), len(query_points), int(bool(exclude_ii)),
                                               _lib.ctypes.byref(h)))
        return cls._from_handle(h)

    def get_ptr(self):
        return self._h

    def copy_c(self, other):
        self.copy(other)

    def copy(self, other=None):
        if other is not None:
            assert isinstance(other, NeighborList)
            h = _lib.ctypes.c_void_p()
            _lib.check(_lib.lib.fg_nlist_copy(other._h, _lib.ctypes.byref(h)))
            self._handle = _lib.Handle(h, _lib.lib.fg_nlist_destroy)
            self._cache = {}
            return self
        new_copy = NeighborList(_null=True)
        new_copy.copy(self)
        return new_copy

    # lists of at least this many bonds come back in page-locked host memory
    _PINNED_BONDS = 1 << 20

    def _arrays(self):
        if "ij" not in self._cache:
            n = len(self)
            empty = _lib.pinned_empty if n >= self._PINNED_BONDS else np.empty
            ij = empty((n, 2), np.uint32)
            d = empty((n,), np.float32)
            v = empty((n, 3), np.float32)
            _lib.check(_lib.lib.fg_nlist_get(self._h, _lib.ptr(ij), _lib.ptr(d), None, _lib.ptr(v)))
            for a in (ij, d, v):
                a.flags.writeable = False
            self._cache.update(ij=ij, d=d, v=v)
        return self._cache

    def __getitem__(self, key):
        return self._arrays()["ij"][key]

    @property
    def query_point_indices(self):
        return self[:, 0]

    @property
    def point_indices(self):
        return self[:, 1]

    @property
    def weights(self):
        if "w" not in self._cache:
            w = np.empty(len(self), np.float32)
            _lib.check(_lib.lib.fg_nlist_get(self._h, None, None, _lib.ptr(w), None))
            w.flags.writeable = False
            self._cache["w"] = w
        return self._cache["w"]

    @property
    def distances(self):
        return self._arrays()["d"]

    @property
    def vectors(self):
        return self._arrays()["v"]

    def _segments(self):
        if "seg" not in self._cache:
            nq = self.num_query_points
            seg = np.zeros(nq, np.uint32)
            cnt = np.zeros(nq, np.uint32)
            _lib.check(_lib.lib.fg_nlist_segments(self._h, _lib.ptr(seg), _lib.ptr(cnt)))
            seg.flags.writeable = False
            cnt.flags.writeable = False
            self._cache.update(seg=seg, cnt=cnt)
        return self._cache

    @property
    def segments(self):
        return self._segments()["seg"]

    @property
    def neighbor_counts(self):
        return self._segments()["cnt"]

    def __len__(self):
        out = _lib.ctypes.c_uint64()
        _lib.check(_lib.lib.fg_nlist_num_bonds(self._h, _lib.ctypes.byref(out)))
        return int(out.value)

    @property
    def num_query_points(self):
        out = _lib.ctypes.c_uint32()
        _lib.check(_lib.lib.fg_nlist_num_query_points(self._h, _lib.ctypes.byref(out)))
        return int(out.value)

    @property
    def num_points(self):
        out = _lib.ctypes.c_uint32()
        _lib.check(_lib.lib.fg_nlist_num_points(self._h, _lib.ctypes.byref(out)))
        return int(out.value)

    def find_first_index(self, i):
        out = _lib.ctypes.c_uint32()
        _lib.check(_lib.lib.fg_nlist_find_first_index(self._h, int(i), _lib.ctypes.byref(out)))
        return int(out.value)

    def filter(self, filt):
        filt = np.ascontiguousarray(filt, dtype=bool).astype(np.uint8)
        _lib.check(_lib.lib.fg_nlist_filter(self._h, _lib.ptr(filt)))
        self._cache = {}
        return self

    def filter_r(self, r_max, r_min=0):
        _lib.check(_lib.lib.fg_nlist_filter_r(self._h, float(r_max), float(r_min)))
        self._cache = {}
        return self

    def sort(self, by_distance=False):
        _lib.check(_lib.lib.fg_nlist_sort(self._h, int(bool(by_distance))))
        self._cache = {}
        return self


def _nlist_from_cnlist(c_nlist):
    return c_nlist


def _make_default_nq(neighbor_query):
    if not isinstance(neighbor_query, NeighborQuery):
        return _RawPoints(*neighbor_query)
    return neighbor_query


def _make_default_nlist(system, neighbors, query_points=None):
    if type(neighbors) is NeighborList:
        return neighbors
    query_args = neighbors.copy()
    query_args.setdefault("exclude_ii", query_points is None)
    nq = _make_default_nq(system)
    qp = query_points if query_points is not None else nq.points
    return nq.query(qp, query_args).toNeighborList()


class _PairCompute(_Compute):
    """Parent of computes that need neighbours (freud/locality.py:924-1000)."""

    def _preprocess_arguments(self, system, query_points=None, neighbors=None):
        nq = NeighborQuery.from_system(system)
        nlist, qargs = self._resolve_neighbors(neighbors, query_points)
        if query_points is None:
            # the system's own points, already on the device (no host copy)
            num_query_points = nq._n_points
        else:
            query_points = _convert_array(query_points, shape=(None, 3))
            num_query_points = query_points.shape[0]
        return (nq, nlist, qargs, query_points, num_query_points)

    def _resolve_neighbors(self, neighbors, query_points=None):
        if type(neighbors) is NeighborList:
            nlist = neighbors
            qargs = _QueryArgs()
        elif neighbors is None or type(neighbors) is dict:
            query_args = self.default_query_args if neighbors is None else neighbors.copy()
            query_args.setdefault("exclude_ii", query_points is None)
            qargs = _QueryArgs.from_dict(query_args)
            nlist = None
        else:
            raise ValueError("An invalid value was provided for neighbors, which must be a dict or NeighborList "
                             "object.")
        return nlist, qargs

    @property
    def default_query_args(self):
        raise NotImplementedError(NO_DEFAULT_QUERY_ARGS_MESSAGE.format(type(self).__name__))


class _SpatialHistogram(_PairCompute):
    """Parent of bond-distance histograms (freud/locality.py:1003-1058)."""

    @property
    def default_query_args(self):
        return dict(mode="ball", r_max=self.r_max)


class _SpatialHistogram1D(_SpatialHistogram):
    pass
