"""The freud-facing API on the GPU, exercised the way freud's own test-suite
exercises it (tests/test_locality_neighbor_query.py, test_locality_neighbor_list.py,
test_density_rdf.py, test_order_steinhardt.py): argument validation and error
classes, mode inference, r_min, reciprocity, exhaustive searches against a numpy
brute force, NeighborList operations, RDF and Steinhardt properties with known
answers."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KINDS = ["aabb", "linkcell", "cellquery"]


def make(freud, kind, box, pts, r_max):
    if kind == "aabb":
        return freud.locality.AABBQuery(box, pts)
    if kind == "linkcell":
        return freud.locality.LinkCell(box, pts, r_max)
    return freud.locality.CellQuery(box, pts)


def neighbours_of(nlist, i):
    return set(int(j) for j in nlist.point_indices[nlist.query_point_indices == i])


def brute_force(box, points, query_points, r_max, r_min=0.0, exclude_ii=False):
    """Pairs within [r_min, r_max) under the minimum image, FP64 numpy."""
    pts = np.asarray(points, np.float64)
    qps = np.asarray(query_points, np.float64)
    out = set()
    for i, q in enumerate(qps):
        d = np.asarray(box.wrap((pts - q).astype(np.float32)), np.float64)
        r = np.sqrt(np.sum(d * d, axis=1))
        for j in np.nonzero((r < r_max) & (r >= r_min))[0]:
            if not (exclude_ii and i == j):
                out.add((i, int(j)))
    return out


# ---- NeighborQuery ---------------------------------------------------------------------

@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("points", [np.zeros((0, 3), np.float32), np.zeros(3, np.float32),
                                    np.zeros((2, 2), np.float32), np.zeros((2, 4), np.float32)])
def test_invalid_points(freud, kind, points):
    with pytest.raises(ValueError):
        make(freud, kind, freud.box.Box.cube(10), points, 2.0)


def test_2d_box_rejects_3d_points(freud):
    pts = np.array([[0, 0, 0], [1, 1, 0.5]], np.float32)
    with pytest.raises(ValueError):
        freud.locality.AABBQuery(freud.box.Box.square(10), pts)


@pytest.mark.parametrize("kind", KINDS)
def test_mode_inference(freud, kind):
    rs = np.random.RandomState(1)
    box = freud.box.Box.cube(9)
    pts = (rs.random_sample((40, 3)) * 9 - 4.5).astype(np.float32)
    nq = make(freud, kind, box, pts, 2.2)
    a = list(nq.query(pts, dict(mode="ball", r_max=2.2, exclude_ii=True)))
    b = list(nq.query(pts, dict(r_max=2.2, exclude_ii=True)))
    assert a == b and len(a) > 0
    if kind != "cellquery":
        a = list(nq.query(pts, dict(mode="nearest", num_neighbors=4)))
        b = list(nq.query(pts, dict(num_neighbors=4)))
        assert a == b and len(a) == 4 * len(pts)


@pytest.mark.parametrize("kind", KINDS)
def test_invalid_query_arguments(freud, kind):
    box = freud.box.Box.cube(10)
    pts = np.zeros((3, 3), np.float32)
    nq = make(freud, kind, box, pts, 2.0)
    with pytest.raises(RuntimeError):
        list(nq.query(pts, dict(mode="ball", num_neighbors=2, r_max=2.0)))
    with pytest.raises(ValueError):
        list(nq.query(pts, dict(r_max=1.0, r_min=1.5)))
    with pytest.raises(ValueError):
        nq.query(pts, dict(r_max=1.0, bogus=3))


@pytest.mark.parametrize("kind", KINDS)
def test_r_min_on_a_line(freud, kind):
    # points at x = 0, 1.5, 2.5, 4 on a line in a big box
    box = freud.box.Box.cube(16)
    pts = np.array([[0, 0, 0], [1.5, 0, 0], [2.5, 0, 0], [4.0, 0, 0]], np.float32)
    nq = make(freud, kind, box, pts, 2.0)
    nl = nq.query(pts, dict(r_max=2.0, r_min=1.2, exclude_ii=True)).toNeighborList()
    assert neighbours_of(nl, 0) == {1}
    assert neighbours_of(nl, 1) == {0}
    assert neighbours_of(nl, 2) == {3}
    assert neighbours_of(nl, 3) == {2}


def test_nearest_with_r_min(freud):
    box = freud.box.Box.cube(16)
    pts = np.array([[0, 0, 0], [1.5, 0, 0], [2.5, 0, 0], [4.0, 0, 0]], np.float32)
    for nq in (freud.locality.AABBQuery(box, pts), freud.locality.LinkCell(box, pts, 2.0)):
        nl = nq.query(pts, dict(num_neighbors=2, r_min=1.2, exclude_ii=True)).toNeighborList()
        assert neighbours_of(nl, 0) == {1, 2}
        assert neighbours_of(nl, 1) == {0, 3}
        assert neighbours_of(nl, 3) == {2, 1}


@pytest.mark.parametrize("kind", KINDS)
def test_reciprocal(freud, kind):
    rs = np.random.RandomState(2)
    box = freud.box.Box(11, 12, 13, 0.2, 0.1, 0.0)
    pts = box.make_absolute(rs.random_sample((500, 3))).astype(np.float32)
    nq = make(freud, kind, box, pts, 2.5)
    nl = nq.query(pts, dict(r_max=2.5, exclude_ii=True)).toNeighborList()
    pairs = set(map(tuple, nl[:].tolist()))
    assert pairs == set((j, i) for i, j in pairs)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_exhaustive_search(freud, kind, seed):
    rs = np.random.RandomState(seed)
    box = freud.box.Box.cube(7.0)
    pts = box.make_absolute(rs.random_sample((250, 3))).astype(np.float32)
    qps = box.make_absolute(rs.random_sample((60, 3))).astype(np.float32)
    nq = make(freud, kind, box, pts, 3.1)
    nl = nq.query(qps, dict(r_max=3.1, r_min=0.2)).toNeighborList()
    got = set(map(tuple, nl[:].tolist()))
    ref = brute_force(box, pts, qps, 3.1, 0.2)
    # float32 pair vectors: pairs within 1e-5 of a bound may fall either way
    boundary = {p for p in got ^ ref}
    for i, j in boundary:
        d = np.linalg.norm(box.wrap((pts[j] - qps[i])[None].astype(np.float32))[0])
        assert min(abs(d - 3.1), abs(d - 0.2)) < 1e-5
    assert len(got ^ ref) <= 2


@pytest.mark.parametrize("kind", KINDS)
def test_no_bonds(freud, kind):
    box = freud.box.Box.cube(20)
    pts = np.array([[0, 0, 0], [5, 5, 5]], np.float32)
    nl = make(freud, kind, box, pts, 1.0).query(pts, dict(r_max=1.0, exclude_ii=True)).toNeighborList()
    assert len(nl) == 0 and nl[:].shape == (0, 2)
    np.testing.assert_array_equal(nl.neighbor_counts, [0, 0])


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("qargs", [dict(r_max=2.0, exclude_ii=False), dict(num_neighbors=4, exclude_ii=False)])
def test_zero_query_points(freud, kind, qargs):
    """A query with an empty (0, 3) array of query points gives an empty list over
    no query points, and the object answers the next query as before."""
    if kind == "cellquery" and "num_neighbors" in qargs:
        pytest.skip("CellQuery answers ball queries only")
    rs = np.random.RandomState(5)
    box = freud.box.Box.cube(10)
    pts = (rs.rand(300, 3) * 10 - 5).astype(np.float32)
    nq = make(freud, kind, box, pts, 2.0)
    nl = nq.query(np.zeros((0, 3), np.float32), qargs).toNeighborList()
    assert len(nl) == 0 and nl[:].shape == (0, 2)
    assert nl.num_query_points == 0 and nl.num_points == 300
    assert nl.neighbor_counts.shape == (0,)
    full = nq.query(pts[:50].copy(), qargs).toNeighborList()
    assert full.num_query_points == 50 and len(full) > 0


@pytest.mark.parametrize("kind", KINDS)
def test_corner_2d(freud, kind):
    # four points near the four corners of a square box are mutual neighbours through the images
    box = freud.box.Box.square(10)
    pts = np.array([[-4.9, -4.9, 0], [4.9, -4.9, 0], [-4.9, 4.9, 0], [4.9, 4.9, 0]], np.float32)
    nl = make(freud, kind, box, pts, 1.0).query(pts, dict(r_max=1.0, exclude_ii=True)).toNeighborList()
    for i in range(4):
        assert neighbours_of(nl, i) == {0, 1, 2, 3} - {i}


def test_linkcell_small_box_shells(freud):
    # fewer than three cells per axis: every neighbour once
    rs = np.random.RandomState(4)
    box = freud.box.Box.cube(5.0)
    pts = box.make_absolute(rs.random_sample((80, 3))).astype(np.float32)
    nl = freud.locality.LinkCell(box, pts, 2.4).query(pts, dict(r_max=2.4, exclude_ii=True)).toNeighborList()
    pairs = nl[:].tolist()
    assert len(pairs) == len(set(map(tuple, pairs)))


@pytest.mark.parametrize("kind", ["aabb", "cellquery"])
def test_too_large_r_max(freud, kind):
    box = freud.box.Box.cube(6.0)
    pts = np.zeros((2, 3), np.float32)
    with pytest.raises(RuntimeError):
        make(freud, kind, box, pts, 3.5).query(pts, dict(r_max=3.5)).toNeighborList()


def test_from_system_and_chaining(freud):
    box = freud.box.Box.cube(10)
    pts = np.random.RandomState(3).random_sample((30, 3)).astype(np.float32) * 10 - 5
    nq = freud.locality.NeighborQuery.from_system((box, pts))
    assert isinstance(nq, freud.locality.NeighborQuery)
    assert freud.locality.NeighborQuery.from_system(nq) is nq
    nl = freud.locality.AABBQuery(box, pts).query(pts, dict(r_max=2.0)).toNeighborList()
    assert len(nl) > 0


# ---- NeighborList ----------------------------------------------------------------------

def sample_nlist(freud, n=300, r_max=2.4, seed=6):
    rs = np.random.RandomState(seed)
    box = freud.box.Box.cube(8.0)
    pts = box.make_absolute(rs.random_sample((n, 3))).astype(np.float32)
    nl = freud.locality.AABBQuery(box, pts).query(pts, dict(r_max=r_max, exclude_ii=True)).toNeighborList()
    return box, pts, nl


def test_nlist_filter_r(freud):
    _, _, nl = sample_nlist(freud)
    d = nl.distances.copy()
    nl2 = nl.copy()
    nl2.filter_r(2.0, 0.5)
    np.testing.assert_array_equal(nl2.distances, d[(d < 2.0) & (d >= 0.5)])
    with pytest.raises(ValueError):
        nl.copy().filter_r(1.0, 2.0)
    with pytest.raises(ValueError):
        nl.copy().filter_r(-1.0)


def test_nlist_filter(freud):
    _, _, nl = sample_nlist(freud)
    ij = nl[:].copy()
    keep = (ij[:, 0] + ij[:, 1]) % 3 == 0
    nl2 = nl.copy()
    nl2.filter(keep)
    np.testing.assert_array_equal(nl2[:], ij[keep])


def test_nlist_segments_counts_first_index(freud):
    _, pts, nl = sample_nlist(freud)
    qi = nl.query_point_indices
    counts = np.bincount(qi, minlength=len(pts))
    np.testing.assert_array_equal(nl.neighbor_counts, counts)
    seg = nl.segments
    for i in (0, 5, 17, len(pts) - 1):
        if counts[i]:
            assert seg[i] == np.searchsorted(qi, i)
            assert nl.find_first_index(i) == np.searchsorted(qi, i)


def test_nlist_from_arrays_and_validation(freud):
    qi = np.array([0, 0, 1, 2, 2], np.uint32)
    pi = np.array([1, 2, 0, 0, 1], np.uint32)
    vec = np.arange(15, dtype=np.float32).reshape(5, 3)
    w = np.array([1, 2, 3, 4, 5], np.float32)
    nl = freud.locality.NeighborList.from_arrays(3, 3, qi, pi, vec, w)
    np.testing.assert_array_equal(nl.query_point_indices, qi)
    np.testing.assert_array_equal(nl.point_indices, pi)
    np.testing.assert_allclose(nl.distances, np.linalg.norm(vec, axis=1), rtol=1e-6)
    np.testing.assert_array_equal(nl.weights, w)
    assert nl.num_query_points == 3 and nl.num_points == 3
    with pytest.raises((ValueError, RuntimeError)):
        freud.locality.NeighborList.from_arrays(3, 3, qi[::-1].copy(), pi, vec)  # not sorted by query index
    with pytest.raises((ValueError, RuntimeError)):
        freud.locality.NeighborList.from_arrays(2, 3, qi, pi, vec)  # query index out of range


def test_nlist_all_pairs(freud):
    box = freud.box.Box.cube(10)
    pts = np.random.RandomState(9).random_sample((12, 3)).astype(np.float32) * 10 - 5
    nl = freud.locality.NeighborList.all_pairs((box, pts))
    assert len(nl) == 12 * 11
    nl = freud.locality.NeighborList.all_pairs((box, pts), query_points=pts[:4], exclude_ii=False)
    assert len(nl) == 4 * 12


def test_nlist_indexing_copy_sort(freud):
    _, _, nl = sample_nlist(freud)
    assert len(nl) == nl[:].shape[0]
    np.testing.assert_array_equal(nl[3], nl[:][3])
    with pytest.raises(IndexError):
        nl[len(nl) + 5]
    c = nl.copy()
    np.testing.assert_array_equal(c[:], nl[:])
    c.sort(by_distance=True)
    qi, d = c.query_point_indices, c.distances
    for i in (0, 3, 8):
        di = d[qi == i]
        assert np.all(np.diff(di) >= 0)
    c.sort()
    np.testing.assert_array_equal(c[:], nl[:])


def test_nlist_default_and_distance_ordering(freud):
    box, pts, nl = sample_nlist(freud, n=150)
    ij = nl[:]
    assert np.all(np.diff(ij[:, 0].astype(np.int64)) >= 0)
    for i in range(0, 150, 13):
        js = ij[ij[:, 0] == i, 1]
        assert np.all(np.diff(js.astype(np.int64)) > 0)
    nl2 = freud.locality.AABBQuery(box, pts).query(pts, dict(r_max=2.4, exclude_ii=True)).toNeighborList(True)
    for i in range(0, 150, 13):
        assert np.all(np.diff(nl2.distances[nl2.query_point_indices == i]) >= 0)


# ---- RDF -------------------------------------------------------------------------------

def test_rdf_bins(freud):
    for r_min in (0.0, 0.5):
        rdf = freud.density.RDF(40, 4.0, r_min)
        edges = rdf.bin_edges
        assert len(edges) == 41 and edges[0] == pytest.approx(r_min) and edges[-1] == pytest.approx(4.0)
        np.testing.assert_allclose(rdf.bin_centers, (edges[1:] + edges[:-1]) / 2, rtol=1e-6)
        assert rdf.bounds == (pytest.approx(r_min), pytest.approx(4.0))
        assert rdf.nbins == 40


def test_rdf_invalid_arguments(freud):
    with pytest.raises(ValueError):
        freud.density.RDF(0, 3.0)
    with pytest.raises(ValueError):
        freud.density.RDF(10, -1.0)
    with pytest.raises(ValueError):
        freud.density.RDF(10, 1.0, 2.0)
    with pytest.raises(ValueError):
        freud.density.RDF(10, 1.0, -0.5)
    with pytest.raises(ValueError):
        freud.density.RDF(10, 1.0, normalization_mode="bogus")


def test_rdf_attribute_access_before_compute(freud):
    rdf = freud.density.RDF(10, 2.0)
    with pytest.raises(AttributeError):
        rdf.rdf


def test_rdf_ideal_gas_and_reset(freud):
    """An ideal gas: g(r) -> 1 and n_r -> rho 4/3 pi r^3; reset=False accumulates."""
    rs = np.random.RandomState(12)
    L, n = 20.0, 16000
    box = freud.box.Box.cube(L)
    pts = (rs.random_sample((n, 3)) * L - L / 2).astype(np.float32)
    rdf = freud.density.RDF(30, 3.0, 0.5)
    rdf.compute((box, pts))
    g = rdf.rdf
    assert np.all(np.abs(g - 1.0) < 0.1)
    r = rdf.bin_edges[1:]
    rho = n / L ** 3
    np.testing.assert_allclose(rdf.n_r[-1], rho * 4 / 3 * np.pi * (r[-1] ** 3 - 0.5 ** 3), rtol=0.05)
    once = rdf.bin_counts.copy()
    rdf.compute((box, pts), reset=False)
    np.testing.assert_array_equal(rdf.bin_counts, 2 * once)
    np.testing.assert_allclose(rdf.rdf, g, rtol=1e-6)
    rdf.compute((box, pts))
    np.testing.assert_array_equal(rdf.bin_counts, once)


def test_rdf_query_points_and_modes(freud):
    rs = np.random.RandomState(13)
    box = freud.box.Box.cube(12.0)
    pts = (rs.random_sample((3000, 3)) * 12 - 6).astype(np.float32)
    qp = pts[:500]
    a = freud.density.RDF(50, 2.5).compute((box, pts), query_points=qp)
    b = freud.density.RDF(50, 2.5, normalization_mode="finite_size").compute((box, pts), query_points=qp)
    np.testing.assert_array_equal(a.bin_counts, b.bin_counts)
    assert not np.array_equal(a.rdf, b.rdf)
    nl = freud.locality.AABBQuery(box, pts).query(qp, dict(r_max=2.5)).toNeighborList()
    c = freud.density.RDF(50, 2.5).compute((box, pts), query_points=qp, neighbors=nl)
    np.testing.assert_array_equal(a.bin_counts, c.bin_counts)


def test_rdf_empty_histogram(freud):
    box = freud.box.Box.cube(30)
    pts = np.array([[0, 0, 0], [10, 10, 10]], np.float32)
    rdf = freud.density.RDF(10, 2.0).compute((box, pts))
    np.testing.assert_array_equal(rdf.bin_counts, 0)
    np.testing.assert_array_equal(rdf.rdf, 0)


def test_rdf_bin_edge_precision(freud):
    # distances exactly on bin edges land in the upper bin, as the reference bins them
    box = freud.box.Box.cube(50)
    pts = np.array([[0, 0, 0], [1.0, 0, 0], [0, 2.0, 0]], np.float32)
    rdf = freud.density.RDF(4, 4.0).compute((box, pts), neighbors=dict(r_max=4.0, exclude_ii=True))
    c = rdf.bin_counts
    assert c[1] == 2 and c[2] == 4  # d = 1 -> bin 1; d = 2 and sqrt(5) -> bin 2


# ---- Steinhardt ------------------------------------------------------------------------

PERFECT_FCC_Q6 = 0.57452416  # tests/test_order_steinhardt.py:17
PERFECT_FCC_W6 = -0.00262604


def perfect_fcc(freud, n=4, a=1.0):
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(*(np.arange(n),) * 3, indexing="ij"), -1).reshape(-1, 3)
    L = n * a
    pts = ((basis[:, None, :] + g[None]).reshape(-1, 3) * a - L / 2 + 0.01).astype(np.float32)
    return freud.box.Box.cube(L), pts


def test_steinhardt_identical_environments(freud):
    box, pts = perfect_fcc(freud)
    st = freud.order.Steinhardt(6)
    st.compute((box, pts), neighbors={"num_neighbors": 12})
    np.testing.assert_allclose(st.ql, PERFECT_FCC_Q6, atol=1e-5)
    np.testing.assert_allclose(st.order, PERFECT_FCC_Q6, atol=1e-5)
    st = freud.order.Steinhardt(6, wl=True, wl_normalize=False)
    st.compute((box, pts), neighbors={"r_max": 0.75})
    np.testing.assert_allclose(st.particle_order, PERFECT_FCC_W6, atol=1e-5)
    st = freud.order.Steinhardt(6, average=True)
    st.compute((box, pts), neighbors={"num_neighbors": 12})
    np.testing.assert_allclose(st.ql, PERFECT_FCC_Q6, atol=1e-5)


def test_steinhardt_shapes_and_properties(freud):
    box, pts = perfect_fcc(freud)
    st = freud.order.Steinhardt([4, 6, 8])
    st.compute((box, pts), neighbors={"num_neighbors": 12})
    assert st.ql.shape == (len(pts), 3)
    assert [q.shape for q in st.particle_harmonics] == [(len(pts), 9), (len(pts), 13), (len(pts), 17)]
    assert st.order.shape == (3,)
    assert st.l == [4, 6, 8] and not st.average and not st.wl
    with pytest.raises(AttributeError):
        freud.order.Steinhardt(6).ql


def test_steinhardt_weighted(freud):
    """Unit weights reproduce the unweighted result; doubling every weight changes nothing."""
    box, pts = perfect_fcc(freud)
    nl = freud.locality.AABBQuery(box, pts).query(pts, dict(num_neighbors=12, exclude_ii=True)).toNeighborList()
    plain = freud.order.Steinhardt(6).compute((box, pts), neighbors=nl).ql
    nl2 = freud.locality.NeighborList.from_arrays(len(pts), len(pts), nl.query_point_indices, nl.point_indices,
                                                  nl.vectors, 2 * np.ones(len(nl), np.float32))
    w = freud.order.Steinhardt(6, weighted=True).compute((box, pts), neighbors=nl2).ql
    np.testing.assert_allclose(w, plain, rtol=1e-5)


def test_steinhardt_rotational_invariance(freud):
    rs = np.random.RandomState(14)
    n = 60
    box = freud.box.Box.cube(40)
    pts = (rs.normal(0, 1.2, (n, 3))).astype(np.float32)
    th = 0.7
    rot = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    rot = rot @ np.array([[1, 0, 0], [0, np.cos(0.4), -np.sin(0.4)], [0, np.sin(0.4), np.cos(0.4)]])
    pr = (pts @ rot.T).astype(np.float32)
    a = freud.order.Steinhardt([4, 6], wl=True).compute((box, pts), neighbors={"num_neighbors": 8})
    b = freud.order.Steinhardt([4, 6], wl=True).compute((box, pr), neighbors={"num_neighbors": 8})
    np.testing.assert_allclose(a.ql, b.ql, rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(a.particle_order, b.particle_order, rtol=1e-3, atol=1e-6)


def test_steinhardt_no_neighbours_gives_nan(freud):
    box = freud.box.Box.cube(30)
    pts = np.array([[0, 0, 0], [10, 10, 10], [10.5, 10, 10]], np.float32)
    st = freud.order.Steinhardt(6).compute((box, pts), neighbors={"r_max": 1.0})
    assert np.isnan(st.ql[0]) and np.all(np.isfinite(st.ql[1:]))


def test_steinhardt_compute_twice(freud):
    box, pts = perfect_fcc(freud)
    st = freud.order.Steinhardt(6)
    a = st.compute((box, pts), neighbors={"num_neighbors": 12}).ql.copy()
    b = st.compute((box, pts), neighbors={"num_neighbors": 12}).ql
    np.testing.assert_array_equal(a, b)


def test_partly_periodic_box_refused(freud):
    """A box that is not periodic on every axis: the reference takes images only
    along periodic axes for a (box, points) system; the cell grids here fold every
    axis, so the query is refused with ValueError instead of answered with folded
    bonds (LinkCell / AABBQuery refuse it as the reference does)."""
    rs = np.random.RandomState(3)
    box = freud.box.Box.cube(10.0)
    box.periodic = [True, True, False]
    pts = box.make_absolute(rs.random_sample((500, 3))).astype(np.float32)
    with pytest.raises(ValueError):
        freud.locality.AABBQuery(box, pts).query(pts, {"r_max": 1.0}).toNeighborList()
    with pytest.raises(ValueError):
        freud.locality.LinkCell(box, pts, 1.0).query(pts, {"r_max": 1.0}).toNeighborList()
    with pytest.raises(ValueError):
        freud.density.RDF(10, 1.0).compute((box, pts))
    with pytest.raises(ValueError):
        freud.order.Steinhardt(6).compute((box, pts), neighbors={"r_max": 1.5})
