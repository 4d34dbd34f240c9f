"""PMFT oracle on the CPU against the fixtures made by the reference's own
PMFTR12.cc / PMFTXYT.cc / PMFTXY.cc / PMFTXYZ.cc (tests/golden/make_pmft_golden.py):
bonds from the oracle's neighbour query, bins in the reference's float arithmetic
with the same C library functions, counts equal; the float32 normalisation
(PMFT.h:70-82, PMFTXYZ.cc:92-104) restated here gives the reference's pcf."""

import numpy as np

from conftest import load_golden
from oracle import oracle as O

f32 = np.float32


def _pcf(kind, counts, maxes, bins, box, n_frames, n_points, n_query, n_equiv=1):
    vol = f32(box[0]) * f32(box[1]) if box[6] else f32(box[0]) * f32(box[1]) * f32(box[2])
    inv_num_dens = f32(vol) / f32(n_query)
    denom = f32(n_frames) * f32(n_points)
    if kind == 3:
        denom = f32(denom * f32(n_equiv))
    prefactor = f32(inv_num_dens * (f32(1.0) / denom))
    c = counts.astype(np.uint32).astype(np.float32)
    if kind == 0:
        dr = f32(maxes[0]) / f32(bins[0])
        product = f32(f32(dr * (f32(2 * np.pi) / f32(bins[1]))) * (f32(1.0) / f32(bins[2])))
        edges = f32(np.arange(bins[0] + 1, dtype=np.float32) * dr)
        r = (edges[:-1] + edges[1:]) / f32(2.0)
        jf = (f32(1.0) / (r * product)).astype(np.float32)[:, None, None]
    else:
        jac = None
        for a in range(3 if kind == 3 else 2):
            d = f32(f32(2.0) * f32(maxes[a])) / f32(bins[a])
            jac = d if jac is None else f32(jac * d)
        if kind == 1:
            jac = f32(jac * (f32(1.0) / f32(bins[2])))
        jf = f32(1.0) / jac
    return ((c * prefactor).astype(np.float32) * jf).astype(np.float32)


def test_pmft_r12_frames():
    g = load_golden("pmft_r12")
    counts = None
    for f in range(int(g["nframes"])):
        box, pts, o = tuple(g["box%d" % f]), g["points%d" % f], g["orient%d" % f]
        ij, d, v = O.query(box, pts, r_max=3.0, exclude_ii=True)
        counts = O.pmft_counts(0, g["maxes"], g["bins"], ij, d, v, p_angle=o, q_angle=o, counts=counts)
    np.testing.assert_array_equal(counts, g["counts"])
    last = int(g["nframes"]) - 1
    n = len(g["points%d" % last])
    pcf = _pcf(0, counts, g["maxes"], g["bins"], tuple(g["box%d" % last]), 2, n, n)
    np.testing.assert_array_equal(pcf, g["pcf"])


def test_pmft_xyt_xy():
    g = load_golden("pmft_xyt")
    box, pts, o = tuple(g["box0"]), g["points0"], g["orient0"]
    ij, d, v = O.query(box, pts, r_max=float(g["r_max"]), exclude_ii=True)
    counts = O.pmft_counts(1, g["maxes"], g["bins"], ij, d, v, p_angle=o, q_angle=o)
    np.testing.assert_array_equal(counts, g["counts"])
    np.testing.assert_array_equal(_pcf(1, counts, g["maxes"], g["bins"], box, 1, len(pts), len(pts)), g["pcf"])
    g = load_golden("pmft_xy")
    box, pts = tuple(g["box0"]), g["points0"]
    qp = g["query_points"]
    ij, d, v = O.query(box, pts, query_points=qp, r_max=float(g["r_max"]), exclude_ii=False)
    counts = O.pmft_counts(2, g["maxes"], g["bins"], ij, d, v, q_angle=g["query_orient"])
    np.testing.assert_array_equal(counts, g["counts"])
    np.testing.assert_array_equal(_pcf(2, counts, g["maxes"], g["bins"], box, 1, len(pts), len(qp)), g["pcf"])


def test_pmft_xyz():
    g = load_golden("pmft_xyz")
    box, pts = tuple(g["box0"]), g["points0"]
    qp = (pts - g["shiftvec"].reshape(1, 3)).astype(np.float32)
    ij, d, v = O.query(box, pts, query_points=qp, r_max=float(g["r_max"]), exclude_ii=True)
    counts = O.pmft_counts(3, g["maxes"], g["bins"], ij, d, v, q_quat=g["query_quats"], equiv=g["equiv"])
    np.testing.assert_array_equal(counts, g["counts"])
    pcf = _pcf(3, counts, g["maxes"], g["bins"], box, 1, len(pts), len(qp), n_equiv=len(g["equiv"]))
    np.testing.assert_array_equal(pcf, g["pcf"])
