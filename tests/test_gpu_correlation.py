"""CorrelationFunction on the GPU against the reference's fixtures
(tests/golden/cf_*.npz, from CorrelationFunction.cc) and the reference's own test
cases (tests/test_density_correlation_function.py). Bin counts must be equal;
the FP64 averages agree with the reference to 1e-12 relative (FP64 sums in a
different order)."""

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-12, 1e-14


def _box(freud, b):
    return freud.box.Box(float(b[0]), float(b[1]), float(b[2]), float(b[3]), float(b[4]), float(b[5]), bool(b[6]))


def test_cf_golden_frames(freud):
    g = load_golden("cf_complex_2d")
    cf = freud.density.CorrelationFunction(int(g["bins"]), float(g["r_max"]))
    for f in range(int(g["nframes"])):
        cf.compute((_box(freud, g["box%d" % f]), g["points%d" % f]), g["values%d" % f], reset=False)
    np.testing.assert_array_equal(cf.bin_counts, g["counts"])
    np.testing.assert_allclose(cf.correlation, g["correlation"], rtol=RTOL, atol=ATOL)
    assert cf.box == _box(freud, g["box1"])


def test_cf_golden_query_points_real(freud):
    g = load_golden("cf_real_query_points")
    cf = freud.density.CorrelationFunction(int(g["bins"]), float(g["r_max"]))
    cf.compute((_box(freud, g["box"]), g["points"]), np.real(g["values"]), g["query_points"],
               np.real(g["query_values"]))
    np.testing.assert_array_equal(cf.bin_counts, g["counts"])
    assert not np.iscomplexobj(cf.correlation)
    np.testing.assert_allclose(cf.correlation, np.real(g["correlation"]), rtol=RTOL, atol=ATOL)


def test_cf_golden_knn_linkcell_nlist(freud):
    g = load_golden("cf_knn")
    box = _box(freud, g["box"])
    cf = freud.density.CorrelationFunction(int(g["bins"]), float(g["r_max"]))
    cf.compute((box, g["points"]), g["values"], neighbors={"num_neighbors": int(g["k"])})
    np.testing.assert_array_equal(cf.bin_counts, g["counts"])
    np.testing.assert_allclose(cf.correlation, g["correlation"], rtol=RTOL, atol=ATOL)
    g = load_golden("cf_linkcell")
    box = _box(freud, g["box"])
    lc = freud.locality.LinkCell(box, g["points"], float(g["cell_width"]))
    cf = freud.density.CorrelationFunction(int(g["bins"]), float(g["r_max"]))
    cf.compute(lc, g["values"])
    np.testing.assert_array_equal(cf.bin_counts, g["counts"])
    np.testing.assert_allclose(cf.correlation, g["correlation"], rtol=RTOL, atol=ATOL)
    # the same bonds as a NeighborList
    nl = lc.query(g["points"], {"r_max": float(g["r_max"]), "exclude_ii": True}).toNeighborList()
    cf2 = freud.density.CorrelationFunction(int(g["bins"]), float(g["r_max"])).compute(lc, g["values"],
                                                                                       neighbors=nl)
    np.testing.assert_array_equal(cf2.bin_counts, g["counts"])
    np.testing.assert_allclose(cf2.correlation, g["correlation"], rtol=RTOL, atol=ATOL)


def test_cf_vs_oracle_large(freud):
    """20 k points, r_max 4: counts equal to the oracle's, averages within 1e-12."""
    rs = np.random.RandomState(90)
    L = 27.0
    box = freud.box.Box.cube(L)
    pts = ((rs.random_sample((20000, 3)) - 0.5) * L).astype(np.float32)
    vals = np.exp(1j * rs.random_sample(20000) * 2 * np.pi) * rs.random_sample(20000)
    qpts = ((rs.random_sample((5000, 3)) - 0.5) * L).astype(np.float32)
    qvals = rs.standard_normal(5000) + 1j * rs.standard_normal(5000)
    cf = freud.density.CorrelationFunction(64, 4.0).compute((box, pts), vals, qpts, qvals)
    b = (L, L, L, 0.0, 0.0, 0.0, 0)
    ij, d, _ = O.query(b, pts, query_points=qpts, r_max=4.0, exclude_ii=False)
    corr, counts, _ = O.correlation(ij, d, vals, qvals, 64, 4.0)
    np.testing.assert_array_equal(cf.bin_counts, counts)
    np.testing.assert_allclose(cf.correlation, corr, rtol=1e-11, atol=1e-14)


def test_cf_query_nn_cases(freud):
    """The reference's nearest-neighbour cases (test_density_correlation_function.py:247-335)."""
    box = freud.box.Box.cube(8)
    points = np.array([[0, 0, 0]], dtype=np.float32)
    query_points = np.array([[0.4, 0.0, 0.0], [0.9, 0.0, 0.0], [0.0, 1.4, 0.0], [0.0, 1.9, 0.0],
                             [0.0, 0.0, 2.4], [0.0, 0.0, 2.9]], dtype=np.float32)
    nn = {"mode": "nearest", "num_neighbors": 1}
    cf = freud.density.CorrelationFunction(3, 3)
    cf.compute((box, points), np.ones(1), query_points, np.ones(6), neighbors=nn)
    np.testing.assert_array_equal(cf.correlation, [1, 1, 1])
    np.testing.assert_array_equal(cf.bin_counts, [2, 2, 2])
    cf.compute((box, query_points), np.ones(6), points, np.ones(1), neighbors=nn)
    np.testing.assert_array_equal(cf.correlation, [1, 0, 0])
    np.testing.assert_array_equal(cf.bin_counts, [1, 0, 0])
    values = [1 + 1j]
    query_values = [1 + 1j, 1 + 1j, 2 + 2j, 2 + 2j, 3 + 3j, 3 + 3j]
    cf.compute((box, points), values, query_points, query_values, neighbors=nn)
    np.testing.assert_array_equal(cf.correlation, [2, 4, 6])
    cf.compute((box, points), np.conj(values), query_points, query_values, neighbors=nn)
    np.testing.assert_array_equal(cf.correlation, [2j, 4j, 6j])
    cf.compute((box, query_points), query_values, points, values, neighbors=nn)
    np.testing.assert_array_equal(cf.correlation, [2, 0, 0])
    cf.compute((box, query_points), np.conj(query_values), points, values, neighbors=nn)
    np.testing.assert_array_equal(cf.correlation, [2j, 0, 0])
    np.testing.assert_array_equal(cf.bin_counts, [1, 0, 0])


def test_cf_attributes_and_errors(freud):
    box, points = freud.data.make_random_system(31.0, 100, is2D=True, seed=1)
    ang = np.random.RandomState(2).random_sample(100) * 2.0 * np.pi
    cf = freud.density.CorrelationFunction(10, 10.0)
    for attr in ("correlation", "box", "bin_counts"):
        with pytest.raises(AttributeError):
            getattr(cf, attr)
    cf.compute((box, points), ang, reset=False)
    assert cf.correlation.dtype == np.float64 and len(cf.bin_counts) == 10
    assert cf.box == box
    cf.compute((box, points), np.exp(1j * ang))
    assert np.iscomplexobj(cf.correlation)
    np.testing.assert_allclose(cf.bin_centers, (np.arange(10) + 0.5), rtol=1e-6)
    assert cf.nbins == 10 and cf.bounds == (0.0, 10.0)
    assert str(cf) == str(eval(repr(cf), {"freud": freud}))
    with pytest.raises(ValueError):
        freud.density.CorrelationFunction(0, 3.0)
    with pytest.raises(ValueError):
        freud.density.CorrelationFunction(10, -1.0)
    with pytest.raises(ValueError):
        cf.compute((box, points), ang[:50])
    with pytest.raises(ValueError):
        cf.compute((box, points), ang, points[:20], ang[:10])
