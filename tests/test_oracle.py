"""CPU tests: the oracle restatement (oracle/freud_oracle.c) is pinned bit for
bit to golden vectors produced by the reference's own CPU sources
(tests/golden/make_golden.py), and its Ylm / Wigner-3j pieces are checked against
scipy / sympy and the reference's known answers."""

import numpy as np
import pytest
from conftest import golden_names, load_golden

from oracle import oracle as O

ARITH = {0: O.ARITH_AABB, 1: O.ARITH_AABB, 2: O.ARITH_WRAP, 3: O.ARITH_GHOST}


@pytest.mark.parametrize("name", golden_names("ball_"))
def test_ball_query_matches_reference(name):
    g = load_golden(name)
    qp = g.get("query_points")
    ij, d, v = O.query(g["box"], g["points"], query_points=qp, r_max=float(g["r_max"]),
                       r_min=float(g.get("r_min", 0.0)), exclude_ii=qp is None, arith=ARITH[int(g["kind"])],
                       sort_by_distance=name.endswith("_bydist"))
    np.testing.assert_array_equal(ij, g["ij"])
    np.testing.assert_array_equal(d, g["d"])
    np.testing.assert_array_equal(v, g["v"])


@pytest.mark.parametrize("name", golden_names("knn_"))
def test_knn_matches_reference(name):
    g = load_golden(name)
    r_max = float(g["r_max"]) if "r_max" in g else -1.0
    excl = name != "knn_aabb_rmax"
    ij, d, v = O.query(g["box"], g["points"], num_neighbors=int(g["k"]), r_max=r_max, exclude_ii=excl,
                       arith=ARITH[int(g["kind"])])
    np.testing.assert_array_equal(ij, g["ij"])
    np.testing.assert_array_equal(d, g["d"])
    np.testing.assert_array_equal(v, g["v"])


def test_rdf_plain_matches_reference():
    g = load_golden("rdf_plain")
    c = O.rdf_counts_query(g["box"], g["points"], int(g["bins"]), float(g["r_max"]))
    np.testing.assert_array_equal(c.astype(np.uint32), g["counts"])
    b = g["box"]
    vol = np.float32(b[0]) * np.float32(b[1]) * np.float32(b[2])
    rdf, nr = O.rdf_reduce(c, float(g["r_max"]), 0.0, 1, len(g["points"]), len(g["points"]), vol)
    np.testing.assert_array_equal(rdf, g["rdf"])
    np.testing.assert_array_equal(nr, g["n_r"])


def test_rdf_cellquery_matches_reference():
    g = load_golden("rdf_cellquery")
    c = O.rdf_counts_query(g["box"], g["points"], int(g["bins"]), float(g["r_max"]), arith=O.ARITH_GHOST)
    np.testing.assert_array_equal(c.astype(np.uint32), g["counts"])


def test_rdf_frames_matches_reference():
    g = load_golden("rdf_frames")
    bins, r_max, r_min = int(g["bins"]), float(g["r_max"]), float(g["r_min"])
    c = np.zeros(bins, np.uint64)
    for f in range(int(g["nframes"])):
        O.rdf_counts_query(g["box%d" % f], g["points%d" % f], bins, r_max, r_min=r_min, counts=c)
    np.testing.assert_array_equal(c.astype(np.uint32), g["counts"])
    last = int(g["nframes"]) - 1
    b = g["box%d" % last]
    vol = np.float32(b[0]) * np.float32(b[1]) * np.float32(b[2])
    n = len(g["points%d" % last])
    rdf, nr = O.rdf_reduce(c, r_max, r_min, int(g["nframes"]), n, n, vol)
    np.testing.assert_array_equal(rdf, g["rdf"])
    np.testing.assert_array_equal(nr, g["n_r"])


def test_rdf_finite_size_matches_reference():
    g = load_golden("rdf_finite_size")
    c = O.rdf_counts_query(g["box"], g["points"], int(g["bins"]), float(g["r_max"]), exclude_ii=False)
    np.testing.assert_array_equal(c.astype(np.uint32), g["counts"])
    b = g["box"]
    vol = np.float32(b[0]) * np.float32(b[1]) * np.float32(b[2])
    n = len(g["points"])
    rdf, nr = O.rdf_reduce(c, float(g["r_max"]), 0.0, 1, n, n, vol, finite_size=True)
    np.testing.assert_array_equal(rdf, g["rdf"])
    np.testing.assert_array_equal(nr, g["n_r"])


def test_bin_edges_match_numpy():
    # reference test_density_rdf.py: bin edges agree with np.histogram_bin_edges
    for bins, r_max, r_min in ((100, 3.0, 0.0), (57, 5.1, 0.3), (500, 5.0, 0.0)):
        e, c = O.bin_edges(bins, r_max, r_min)
        np.testing.assert_allclose(e, np.histogram_bin_edges([], bins, (r_min, r_max)), rtol=1e-5, atol=1e-6)


def test_ylm_matches_scipy():
    special = pytest.importorskip("scipy.special")
    rng = np.random.default_rng(0)
    for l in range(0, 13):
        for _ in range(5):
            th, ph = rng.uniform(0, np.pi), rng.uniform(-np.pi, np.pi)
            ms = list(range(0, l + 1)) + [-m for m in range(1, l + 1)]
            ref = np.array([special.sph_harm_y(l, m, th, ph) for m in ms])
            np.testing.assert_allclose(O.ylm(l, th, ph), ref, rtol=1e-12, atol=1e-13)


def test_wigner3j_matches_sympy():
    wigner = pytest.importorskip("sympy.physics.wigner")
    for l in (2, 4, 6, 12):
        for m1, m2 in ((0, 0), (1, -1), (2, -3), (l, -l), (-1, 2)):
            m3 = -m1 - m2
            if abs(m2) > l or abs(m3) > l:
                continue
            ref = float(wigner.wigner_3j(l, l, l, m1, m2, m3))
            assert abs(O.wigner3j(l, m1, m2, m3) - ref) < 1e-12


@pytest.mark.parametrize("name", golden_names("st_"))
def test_steinhardt_matches_reference(name):
    g = load_golden(name)
    ls = g["ls"]
    if "r_max" in g:
        ij, d, v = O.query(g["box"], g["points"], r_max=float(g["r_max"]), exclude_ii=True)
    else:
        ij, d, v = O.query(g["box"], g["points"], num_neighbors=12, exclude_ii=True)
    av, wl = bool(g.get("average", 0)), bool(g.get("wl", 0))
    o = O.steinhardt(ls, g["box"], g["points"], ij, d, average=av, wl=wl, wl_normalize=bool(g.get("wl_normalize", 0)))
    ql = o["ql_ave"] if av else o["ql"]
    np.testing.assert_allclose(ql, g["ql"], rtol=2e-5, atol=2e-6)
    po = o["wl"] if wl else ql
    scale = np.max(np.abs(po), axis=0)
    # the reference's float32 Wl (fsph harmonics, plain float triple sums) is within
    # 5.6e-6 of the |w| scale of FP64 on these inputs (W10 of the kNN case)
    assert np.all(np.abs(po - g["particle_order"]) <= 2e-5 * scale + 1e-7)
    np.testing.assert_allclose(o["order"], g["order"], rtol=5e-5, atol=1e-6)
    qlm = np.concatenate([q.reshape(-1) for q in o["qlm"]])
    np.testing.assert_allclose(qlm, g["qlm"], atol=5e-6)


def test_perfect_fcc_q6_known_answer():
    # reference test_order_steinhardt.py:17-18 PERFECT_FCC_Q6 = 0.57452416
    from golden.make_golden import fcc

    box, pts = fcc(4, 1.5874, 0.0, 0)
    ij, d, v = O.query(box, pts, num_neighbors=12, exclude_ii=True)
    o = O.steinhardt([6], box, pts, ij, d)
    np.testing.assert_allclose(o["ql"][:, 0], 0.57452416, atol=1e-5)
    np.testing.assert_allclose(o["order"][0], 0.57452416, atol=1e-5)
