"""ctypes wrapper around oracle/_ref/libfreud_ref.so (the reference's own CPU
sources compiled in place by oracle/build_ref.sh).

TEST INFRASTRUCTURE ONLY: used to generate golden vectors and to pin the oracle
restatement. The library exists only where the reference sources are present
(it is built for the host it was compiled on), so callers must check
``available()``.
"""

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "libfreud_ref.so")
_lib = None

KIND_RAW, KIND_AABB, KIND_LINKCELL, KIND_CELLQUERY = 0, 1, 2, 3
MODE_INFER, MODE_BALL, MODE_NEAREST = 0, 1, 2
DEFAULT_NUM_NEIGHBORS = 0xFFFFFFFF


class RefError(Exception):
    def __init__(self, cls, msg):
        super().__init__(msg)
        self.cls = cls


def available():
    return _load() is not None


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        return None
    try:
        lib = ctypes.CDLL(_LIB_PATH)
    except OSError:
        return None
    P = ctypes.c_void_p
    f32, u32, i32 = ctypes.c_float, ctypes.c_uint, ctypes.c_int
    lib.ref_query.restype = P
    lib.ref_query.argtypes = [i32, P, i32, P, u32, f32, P, u32, i32, u32, f32, f32,
                              f32, f32, i32, i32, P, P, ctypes.c_char_p, i32]
    lib.ref_nlist_copy.argtypes = [P, P, P, P, P]
    lib.ref_nlist_free.argtypes = [P]
    lib.ref_rdf.restype = i32
    lib.ref_rdf.argtypes = [u32, f32, f32, i32, i32, P, P, P, P, i32, f32, i32, u32, f32,
                            f32, i32, P, P, P, P, P, P, P, ctypes.c_char_p, i32]
    lib.ref_pmft.restype = i32
    lib.ref_pmft.argtypes = [i32, P, P, i32, P, P, P, P, P, P, P, P, P, u32, i32, i32, u32, f32, f32, i32, P, P,
                             ctypes.c_char_p, i32]
    lib.ref_cf.restype = i32
    lib.ref_cf.argtypes = [u32, f32, i32, P, P, P, P, P, P, P, P, i32, f32, i32, u32, f32, f32, i32, P, P,
                           ctypes.c_char_p, i32]
    lib.ref_steinhardt.restype = i32
    lib.ref_steinhardt.argtypes = [P, u32, i32, i32, i32, i32, P, i32, P, u32, i32, f32,
                                   i32, u32, f32, f32, i32, i32, u32, P, P, P, P, P, P,
                                   P, ctypes.c_char_p, i32]
    _lib = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _box6(box):
    """box: (Lx, Ly, Lz, xy, xz, yz, is2D)."""
    return np.asarray(box[:6], dtype=np.float32), int(box[6])


def query(kind, box, points, query_points, mode=MODE_INFER, num_neighbors=DEFAULT_NUM_NEIGHBORS,
          r_max=-1.0, r_min=0.0, r_guess=-1.0, scale=-1.0, exclude_ii=False, cell_width=0.0,
          sort_by_distance=False):
    """Returns (ij (B,2) uint32, distances, weights, vectors (B,3))."""
    lib = _load()
    b6, is2d = _box6(box)
    pts = np.ascontiguousarray(points, dtype=np.float32)
    qp = np.ascontiguousarray(query_points, dtype=np.float32)
    nb = ctypes.c_uint(0)
    st = ctypes.c_int(0)
    err = ctypes.create_string_buffer(512)
    h = lib.ref_query(kind, _ptr(b6), is2d, _ptr(pts), len(pts), cell_width, _ptr(qp), len(qp), mode,
                      num_neighbors, r_max, r_min, r_guess, scale, int(exclude_ii),
                      int(sort_by_distance), ctypes.byref(nb), ctypes.byref(st), err, 512)
    if st.value != 0:
        raise RefError(st.value, err.value.decode())
    n = nb.value
    ij = np.zeros((n, 2), np.uint32)
    d = np.zeros(n, np.float32)
    w = np.zeros(n, np.float32)
    v = np.zeros((n, 3), np.float32)
    lib.ref_nlist_copy(h, _ptr(ij), _ptr(d), _ptr(w), _ptr(v))
    lib.ref_nlist_free(h)
    return ij, d, w, v


def rdf(bins, r_max, frames, r_min=0.0, finite_size=False, kind=KIND_RAW, cell_width=0.0,
        mode=MODE_BALL, num_neighbors=DEFAULT_NUM_NEIGHBORS, q_r_max=None, q_r_min=0.0,
        exclude_ii=True, nlists=None):
    """frames: list of (box, points). nlists: optional list of (ij, vectors, weights).
    Returns (counts uint32, rdf float32, n_r float32)."""
    lib = _load()
    boxes = np.concatenate([_box6(b)[0] for b, _ in frames]).astype(np.float32)
    is2d = np.array([int(b[6]) for b, _ in frames], np.int32)
    sizes = [len(p) for _, p in frames]
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    pts = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float32) for _, p in frames]))
    nbpf = ij = vec = w = None
    if nlists is not None:
        nbpf = np.array([len(x[0]) for x in nlists], np.uint32)
        ij = np.ascontiguousarray(np.concatenate([x[0] for x in nlists]).astype(np.uint32))
        vec = np.ascontiguousarray(np.concatenate([x[1] for x in nlists]).astype(np.float32))
        w = np.ascontiguousarray(np.concatenate([x[2] for x in nlists]).astype(np.float32))
    counts = np.zeros(bins, np.uint32)
    g = np.zeros(bins, np.float32)
    nr = np.zeros(bins, np.float32)
    err = ctypes.create_string_buffer(512)
    st = lib.ref_rdf(bins, r_max, r_min, int(finite_size), len(frames), _ptr(boxes), _ptr(is2d),
                     _ptr(offsets), _ptr(pts), kind, cell_width, mode, num_neighbors,
                     r_max if q_r_max is None else q_r_max, q_r_min, int(exclude_ii), _ptr(nbpf),
                     _ptr(ij), _ptr(vec), _ptr(w), _ptr(counts), _ptr(g), _ptr(nr), err, 512)
    if st != 0:
        raise RefError(st, err.value.decode())
    return counts, g, nr


def cf(bins, r_max, frames, values, query_frames=None, query_values=None, kind=KIND_RAW, cell_width=0.0,
       mode=MODE_BALL, num_neighbors=DEFAULT_NUM_NEIGHBORS, q_r_max=None, q_r_min=0.0, exclude_ii=True):
    """CorrelationFunction over frames (list of (box, points)) with per-frame values
    (list of complex arrays); query_frames: per-frame query points (None: the
    points). Returns (counts uint32, correlation complex128)."""
    lib = _load()
    boxes = np.concatenate([_box6(b)[0] for b, _ in frames]).astype(np.float32)
    is2d = np.array([int(b[6]) for b, _ in frames], np.int32)
    offsets = np.concatenate([[0], np.cumsum([len(p) for _, p in frames])]).astype(np.uint32)
    pts = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float32) for _, p in frames]))
    vals = np.ascontiguousarray(np.concatenate([np.asarray(v, np.complex128) for v in values]))
    qoff = qpts = qvals = None
    if query_frames is not None:
        qoff = np.concatenate([[0], np.cumsum([len(q) for q in query_frames])]).astype(np.uint32)
        qpts = np.ascontiguousarray(np.concatenate([np.asarray(q, np.float32) for q in query_frames]))
        if query_values is not None:
            qvals = np.ascontiguousarray(np.concatenate([np.asarray(v, np.complex128) for v in query_values]))
    counts = np.zeros(bins, np.uint32)
    corr = np.zeros(bins, np.complex128)
    err = ctypes.create_string_buffer(512)
    st = lib.ref_cf(bins, r_max, len(frames), _ptr(boxes), _ptr(is2d), _ptr(offsets), _ptr(pts), _ptr(vals),
                    _ptr(qoff), _ptr(qpts), _ptr(qvals), kind, cell_width, mode, num_neighbors,
                    r_max if q_r_max is None else q_r_max, q_r_min, int(exclude_ii), _ptr(counts), _ptr(corr),
                    err, 512)
    if st != 0:
        raise RefError(st, err.value.decode())
    return counts, corr


def pmft(kind, maxes, bins, frames, orientations=None, query_frames=None, query_orientations=None,
         equiv=None, nq_kind=KIND_RAW, mode=MODE_BALL, num_neighbors=DEFAULT_NUM_NEIGHBORS, r_max=-1.0,
         r_min=0.0, exclude_ii=True):
    """PMFT (kind 0 R12, 1 XYT, 2 XY, 3 XYZ) over frames (list of (box, points)).
    orientations / query_orientations: per-frame lists (angles, or (n, 4)
    quaternions for XYZ). Returns (counts uint32, pcf float32) shaped by bins."""
    lib = _load()
    boxes = np.concatenate([_box6(b)[0] for b, _ in frames]).astype(np.float32)
    is2d = np.array([int(b[6]) for b, _ in frames], np.int32)
    offsets = np.concatenate([[0], np.cumsum([len(p) for _, p in frames])]).astype(np.uint32)
    pts = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float32) for _, p in frames]))
    cat = (lambda xs: None if xs is None else np.ascontiguousarray(np.concatenate(
        [np.asarray(x, np.float32).reshape(len(x), -1) for x in xs]), np.float32))
    orient = cat(orientations)
    qoff = qpts = None
    if query_frames is not None:
        qoff = np.concatenate([[0], np.cumsum([len(q) for q in query_frames])]).astype(np.uint32)
        qpts = np.ascontiguousarray(np.concatenate([np.asarray(q, np.float32) for q in query_frames]))
    qorient = cat(query_orientations)
    eq = None if equiv is None else np.ascontiguousarray(equiv, np.float32)
    m = np.asarray(maxes, np.float32)
    b = np.asarray(bins, np.uint32)
    n = int(np.prod(b))
    counts = np.zeros(n, np.uint32)
    pcf = np.zeros(n, np.float32)
    err = ctypes.create_string_buffer(512)
    st = lib.ref_pmft(int(kind), _ptr(m), _ptr(b), len(frames), _ptr(boxes), _ptr(is2d), _ptr(offsets), _ptr(pts),
                      _ptr(orient), _ptr(qoff), _ptr(qpts), _ptr(qorient), _ptr(eq), 0 if eq is None else len(eq),
                      nq_kind, mode, num_neighbors, r_max, r_min, int(exclude_ii), _ptr(counts), _ptr(pcf), err,
                      512)
    if st != 0:
        raise RefError(st, err.value.decode())
    return counts.reshape(tuple(int(x) for x in b)), pcf.reshape(tuple(int(x) for x in b))


def steinhardt(ls, box, points, average=False, wl=False, weighted=False, wl_normalize=False,
               kind=KIND_RAW, cell_width=0.0, mode=MODE_INFER, num_neighbors=DEFAULT_NUM_NEIGHBORS,
               r_max=-1.0, r_min=0.0, exclude_ii=True, nlist=None):
    """Returns dict with ql (N, nl), particle_order (N, nl), qlm (list per l of (N, 2l+1)
    complex64) and order (nl,)."""
    lib = _load()
    ls = np.asarray(np.atleast_1d(ls), np.uint32)
    b6, is2d = _box6(box)
    pts = np.ascontiguousarray(points, np.float32)
    n = len(pts)
    nl = len(ls)
    stride = int(np.sum(2 * ls + 1))
    ql = np.zeros((n, nl), np.float32)
    po = np.zeros((n, nl), np.float32)
    qlm = np.zeros((n, stride, 2), np.float32)
    order = np.zeros(nl, np.float32)
    ij = vec = w = None
    nb = 0
    if nlist is not None:
        ij = np.ascontiguousarray(nlist[0], np.uint32)
        vec = np.ascontiguousarray(nlist[1], np.float32)
        w = np.ascontiguousarray(nlist[2], np.float32)
        nb = len(ij)
    err = ctypes.create_string_buffer(512)
    st = lib.ref_steinhardt(_ptr(ls), nl, int(average), int(wl), int(weighted), int(wl_normalize),
                            _ptr(b6), is2d, _ptr(pts), n, kind, cell_width, mode, num_neighbors,
                            r_max, r_min, int(exclude_ii), int(nlist is not None), nb, _ptr(ij),
                            _ptr(vec), _ptr(w), _ptr(ql), _ptr(po), _ptr(qlm), _ptr(order), err, 512)
    if st != 0:
        raise RefError(st, err.value.decode())
    qc = qlm[..., 0] + 1j * qlm[..., 1]
    out, off = [], 0
    for l in ls:
        out.append(qc[:, off:off + 2 * l + 1].astype(np.complex64))
        off += 2 * l + 1
    return {"ql": ql, "particle_order": po, "qlm": out, "order": order}
