"""ctypes wrapper for the CPU oracle (oracle/freud_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker / baseline, never as part
of the product. ``build()`` compiles the C restatement with gcc (no FMA
contraction, so float32 results are bit-identical to the reference's x86 build).
"""

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "freud_oracle.c")
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

ARITH_AABB, ARITH_WRAP, ARITH_GHOST = 0, 1, 2


def build(force=False):
    """Compile liboracle.so if missing or older than its source."""
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        tmp = _LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, _SRC,
                               "-lm", "-lpthread"])
        os.replace(tmp, _LIB)
    return _LIB


def _load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(_LIB)
    P = ctypes.c_void_p
    u32, u64, f32, i32 = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float, ctypes.c_int
    lib.ofg_query.restype = i32
    lib.ofg_query.argtypes = [P, P, u32, P, u32, u32, f32, f32, i32, i32, i32, i32, P, P]
    lib.ofg_nlist_copy.argtypes = [P, P, P, P]
    lib.ofg_nlist_free.argtypes = [P]
    lib.ofg_rdf_query.restype = i32
    lib.ofg_rdf_query.argtypes = [P, P, u32, P, u32, f32, f32, i32, i32, u32, f32, f32, i32, P]
    lib.ofg_hist.argtypes = [P, u64, u32, f32, f32, P]
    lib.ofg_bin_index.argtypes = [P, u64, u32, f32, f32, P]
    lib.ofg_pmft.argtypes = [ctypes.c_int, u64, P, P, P, P, P, P, P, u32, P, P]
    lib.ofg_bin_edges.argtypes = [u32, f32, f32, P, P]
    lib.ofg_rdf_reduce.argtypes = [P, u32, f32, f32, u32, u32, u32, f32, i32, i32, P, P]
    lib.ofg_ylm.argtypes = [i32, ctypes.c_double, ctypes.c_double, P]
    lib.ofg_wigner3j.restype = ctypes.c_double
    lib.ofg_wigner3j.argtypes = [i32, i32, i32, i32]
    lib.ofg_steinhardt.restype = i32
    lib.ofg_steinhardt.argtypes = [P, u32, i32, i32, i32, i32, P, P, u32, u64, P, P, P, P, P, P, P, P, P, i32]
    lib.ofg_box_wrap.argtypes = [P, P, u64, P]
    lib.ofg_box_fractional.argtypes = [P, P, u64, P]
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def box7(box):
    """(Lx, Ly, Lz, xy, xz, yz, is2D) as float32[7] from a tuple or a Box-like object."""
    if hasattr(box, "Lx"):
        return np.array([box.Lx, box.Ly, box.Lz, box.xy, box.xz, box.yz, 1.0 if box.is2D else 0.0],
                        np.float32)
    return np.asarray(box, np.float32).reshape(7)


def default_threads():
    return os.cpu_count() or 1


def query(box, points, query_points=None, r_max=-1.0, r_min=0.0, num_neighbors=0, exclude_ii=False,
          arith=ARITH_AABB, sort_by_distance=False, threads=None):
    """NeighborList in reference order. num_neighbors > 0 selects kNN. Returns
    (ij (B,2) uint32, distances (B,) float32, vectors (B,3) float32)."""
    lib = _load()
    b = box7(box)
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    qp = pts if query_points is None else np.ascontiguousarray(query_points, np.float32).reshape(-1, 3)
    if r_max is None or r_max < 0:
        r_max = np.inf
    nb = ctypes.c_uint64(0)
    h = ctypes.c_void_p(0)
    lib.ofg_query(_p(b), _p(pts), len(pts), _p(qp), len(qp), int(num_neighbors), float(r_max), float(r_min),
                  int(exclude_ii), int(arith), int(sort_by_distance), threads or default_threads(),
                  ctypes.byref(nb), ctypes.byref(h))
    n = nb.value
    ij = np.zeros((n, 2), np.uint32)
    d = np.zeros(n, np.float32)
    v = np.zeros((n, 3), np.float32)
    lib.ofg_nlist_copy(h, _p(ij), _p(d), _p(v))
    lib.ofg_nlist_free(h)
    return ij, d, v


def rdf_counts_query(box, points, bins, r_max, r_min=0.0, query_points=None, exclude_ii=True,
                     arith=ARITH_AABB, counts=None, threads=None):
    """Fused ball query + histogram; adds into and returns uint64 counts."""
    lib = _load()
    b = box7(box)
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    qp = pts if query_points is None else np.ascontiguousarray(query_points, np.float32).reshape(-1, 3)
    if counts is None:
        counts = np.zeros(bins, np.uint64)
    lib.ofg_rdf_query(_p(b), _p(pts), len(pts), _p(qp), len(qp), float(r_max), 0.0, int(exclude_ii),
                      int(arith), int(bins), float(r_min), float(r_max), threads or default_threads(),
                      _p(counts))
    return counts


def hist(distances, bins, r_max, r_min=0.0, counts=None):
    lib = _load()
    d = np.ascontiguousarray(distances, np.float32)
    if counts is None:
        counts = np.zeros(bins, np.uint64)
    lib.ofg_hist(_p(d), len(d), int(bins), float(r_min), float(r_max), _p(counts))
    return counts


def bin_index(distances, bins, r_max, r_min=0.0):
    """Histogram bin of each distance (int64, -1 when outside [r_min, r_max))."""
    lib = _load()
    d = np.ascontiguousarray(distances, np.float32)
    out = np.zeros(len(d), np.int64)
    lib.ofg_bin_index(_p(d), len(d), int(bins), float(r_min), float(r_max), _p(out))
    return out


def correlation(ij, distances, values, query_values, bins, r_max, sums=None, counts=None):
    """CorrelationFunction accumulate + reduce (CorrelationFunction.cc:48-59, 79-96)
    over given bonds: per bin, the count and the FP64 sum of conj(values[j]) *
    query_values[i]. Adds into (sums, counts) when given; returns
    (correlation, counts, sums), correlation = sums / counts where counts != 0."""
    ij = np.asarray(ij, np.int64).reshape(-1, 2)
    k = bin_index(distances, bins, r_max)
    keep = k >= 0
    v = np.asarray(values, np.complex128)
    q = np.asarray(query_values, np.complex128)
    prod = np.conj(v[ij[keep, 1]]) * q[ij[keep, 0]]
    if sums is None:
        sums = np.zeros(bins, np.complex128)
    if counts is None:
        counts = np.zeros(bins, np.uint64)
    np.add.at(sums, k[keep], prod)
    np.add.at(counts, k[keep], 1)
    corr = sums.copy()
    nz = counts != 0
    corr[nz] = sums[nz] / counts[nz].astype(np.float64)
    return corr, counts, sums


PMFT_AXES = {
    0: lambda m, b: [(0.0, m[0], b[0]), (0.0, 2 * np.pi, b[1]), (0.0, 2 * np.pi, b[2])],
    1: lambda m, b: [(-m[0], m[0], b[0]), (-m[1], m[1], b[1]), (0.0, 2 * np.pi, b[2])],
    2: lambda m, b: [(-m[0], m[0], b[0]), (-m[1], m[1], b[1]), (0.0, 1.0, 1)],
    3: lambda m, b: [(-m[0], m[0], b[0]), (-m[1], m[1], b[1]), (-m[2], m[2], b[2])],
}


def pmft_counts(kind, maxes, bins, ij, distances, vectors, p_angle=None, q_angle=None, q_quat=None, equiv=None,
                counts=None):
    """PMFT bin counts (kind 0 R12, 1 XYT, 2 XY, 3 XYZ) of a list's bonds, in the
    reference's float arithmetic (PMFT*.cc accumulate). Adds into and returns
    uint64 counts shaped by bins (XY: (n_x, n_y))."""
    lib = _load()
    axes = np.array([[np.float32(a), np.float32(b), np.float32(n)] for a, b, n in
                     PMFT_AXES[kind](list(maxes), list(bins))], np.float32).reshape(-1)
    shape = tuple(int(x) for x in bins)
    n = int(np.prod(shape))
    if counts is None:
        counts = np.zeros(n, np.uint64)
    c = np.ascontiguousarray(counts.reshape(-1))
    ijc = np.ascontiguousarray(ij, np.uint32).reshape(-1, 2)
    d = np.ascontiguousarray(distances, np.float32)
    v = np.ascontiguousarray(vectors, np.float32).reshape(-1, 3)
    conv = (lambda a: None if a is None else np.ascontiguousarray(a, np.float32))
    eq = conv(equiv)
    lib.ofg_pmft(int(kind), len(d), _p(ijc), _p(d), _p(v), _p(conv(p_angle)), _p(conv(q_angle)), _p(conv(q_quat)),
                 _p(eq), 0 if eq is None else len(eq), _p(axes), _p(c))
    return c.reshape(shape)


def bin_edges(bins, r_max, r_min=0.0):
    lib = _load()
    e = np.zeros(bins + 1, np.float32)
    c = np.zeros(bins + 1, np.float32)
    lib.ofg_bin_edges(int(bins), float(r_min), float(r_max), _p(e), _p(c))
    return e, c[:bins]


def rdf_reduce(counts, r_max, r_min, n_frames, n_points, n_query_points, volume, is2d=False,
               finite_size=False):
    """float32 (rdf, n_r) from uint32 counts, as the reference normalises them."""
    lib = _load()
    c = np.ascontiguousarray(np.asarray(counts).astype(np.uint32))
    bins = len(c)
    g = np.zeros(bins, np.float32)
    nr = np.zeros(bins, np.float32)
    lib.ofg_rdf_reduce(_p(c), bins, float(r_min), float(r_max), int(n_frames), int(n_points),
                       int(n_query_points), float(np.float32(volume)), int(is2d), int(finite_size), _p(g),
                       _p(nr))
    return g, nr


def ylm(l, theta, phi):
    lib = _load()
    out = np.zeros(2 * (2 * l + 1))
    lib.ofg_ylm(int(l), float(theta), float(phi), _p(out))
    return out[0::2] + 1j * out[1::2]


def wigner3j(l, m1, m2, m3):
    return _load().ofg_wigner3j(int(l), int(m1), int(m2), int(m3))


def steinhardt(ls, box, points, ij, distances, weights=None, average=False, wl=False, weighted=False,
               wl_normalize=False, threads=None):
    """FP64 Steinhardt over a NeighborList sorted by query index. Returns a dict with
    ql, ql_ave, wl (N, nl) float64, wl_mag (N, nl) = sum of |Wigner-3j terms| (the
    scale of the cancellation in w_l), qlm list of (N, 2l+1) complex128, order (nl,)."""
    lib = _load()
    ls = np.asarray(np.atleast_1d(ls), np.uint32)
    b = box7(box)
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    n = len(pts)
    nl = len(ls)
    stride = int(np.sum(2 * ls + 1))
    ij = np.ascontiguousarray(ij, np.uint32).reshape(-1, 2)
    d = np.ascontiguousarray(distances, np.float32)
    w = np.ascontiguousarray(np.ones(len(d), np.float32) if weights is None else weights, np.float32)
    ql = np.zeros((n, nl))
    qla = np.zeros((n, nl))
    wlo = np.zeros((n, nl))
    qlm = np.zeros((n, stride, 2))
    order = np.zeros(nl)
    wmag = np.zeros((n, nl))
    lib.ofg_steinhardt(_p(ls), nl, int(average), int(wl), int(weighted), int(wl_normalize), _p(b), _p(pts), n,
                       len(d), _p(ij), _p(d), _p(w), _p(ql), _p(qla), _p(wlo), _p(qlm), _p(order), _p(wmag),
                       int(threads or default_threads()))
    qc = qlm[..., 0] + 1j * qlm[..., 1]
    out, off = [], 0
    for l in ls:
        out.append(qc[:, off:off + 2 * l + 1])
        off += 2 * l + 1
    return {"ql": ql, "ql_ave": qla, "wl": wlo, "wl_mag": wmag, "qlm": out, "order": order}


def box_wrap(box, vecs):
    lib = _load()
    b = box7(box)
    v = np.ascontiguousarray(vecs, np.float32).reshape(-1, 3)
    out = np.zeros_like(v)
    lib.ofg_box_wrap(_p(b), _p(v), len(v), _p(out))
    return out
