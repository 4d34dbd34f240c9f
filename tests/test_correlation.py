"""CorrelationFunction oracle on the CPU: bonds from the oracle's neighbour
query, exact bin indices, FP64 sums of conj(values[j]) * query_values[i], against
the fixtures made by the reference's own CorrelationFunction.cc
(tests/golden/make_cf_golden.py). Counts must be equal; the FP64 averages agree
to 1e-12 relative (the summation order differs from the reference's threads)."""

import numpy as np

from conftest import load_golden
from oracle import oracle as O

RTOL, ATOL = 1e-12, 1e-14


def _frame_sums(box, pts, values, bins, hist_max, qpts=None, qvalues=None, sums=None, counts=None, **q):
    ij, d, _ = O.query(box, pts, query_points=qpts, **q)
    return O.correlation(ij, d, values, values if qvalues is None else qvalues, bins, hist_max, sums, counts)


def test_cf_complex_2d_frames():
    g = load_golden("cf_complex_2d")
    bins, r_max = int(g["bins"]), float(g["r_max"])
    sums = counts = None
    for f in range(int(g["nframes"])):
        corr, counts, sums = _frame_sums(tuple(g["box%d" % f]), g["points%d" % f], g["values%d" % f], bins, r_max,
                                         sums=sums, counts=counts, r_max=r_max, exclude_ii=True)
    np.testing.assert_array_equal(counts, g["counts"])
    np.testing.assert_allclose(corr, g["correlation"], rtol=RTOL, atol=ATOL)


def test_cf_query_points():
    g = load_golden("cf_real_query_points")
    bins, r_max = int(g["bins"]), float(g["r_max"])
    corr, counts, _ = _frame_sums(tuple(g["box"]), g["points"], g["values"], bins, r_max, qpts=g["query_points"],
                                  qvalues=g["query_values"], r_max=r_max, exclude_ii=False)
    np.testing.assert_array_equal(counts, g["counts"])
    np.testing.assert_allclose(corr, g["correlation"], rtol=RTOL, atol=ATOL)


def test_cf_knn_and_linkcell():
    g = load_golden("cf_knn")
    corr, counts, _ = _frame_sums(tuple(g["box"]), g["points"], g["values"], int(g["bins"]), float(g["r_max"]),
                                  num_neighbors=int(g["k"]), exclude_ii=True)
    np.testing.assert_array_equal(counts, g["counts"])
    np.testing.assert_allclose(corr, g["correlation"], rtol=RTOL, atol=ATOL)
    g = load_golden("cf_linkcell")
    r_max = float(g["r_max"])
    corr, counts, _ = _frame_sums(tuple(g["box"]), g["points"], g["values"], int(g["bins"]), r_max, r_max=r_max,
                                  exclude_ii=True, arith=O.ARITH_WRAP)
    np.testing.assert_array_equal(counts, g["counts"])
    np.testing.assert_allclose(corr, g["correlation"], rtol=RTOL, atol=ATOL)
