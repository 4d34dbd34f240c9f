"""GPU parity: the CUDA path through the C ABI against the reference's golden
vectors and the oracle. Neighbour sets, distances, vectors and RDF counts are
compared bit for bit; Steinhardt within the tolerances written in each test."""

import numpy as np
import pytest
from conftest import golden_names, load_golden

from oracle import oracle as O

pytestmark = pytest.mark.gpu

KIND_CLASS = {0: "_RawPoints", 1: "AABBQuery", 2: "LinkCell", 3: "CellQuery"}
ARITH = {0: O.ARITH_AABB, 1: O.ARITH_AABB, 2: O.ARITH_WRAP, 3: O.ARITH_GHOST}


def box_of(freud, b):
    return freud.box.Box(float(b[0]), float(b[1]), float(b[2]), float(b[3]), float(b[4]), float(b[5]), bool(b[6]))


def make_nq(freud, kind, box, pts, cell_width=0.0):
    if kind == 3:
        return freud.locality.CellQuery(box, pts)
    if kind == 2:
        return freud.locality.LinkCell(box, pts, cell_width)
    if kind == 1:
        return freud.locality.AABBQuery(box, pts)
    return freud.locality._RawPoints(box, pts)


def assert_nlist_equal(nl, ij, d, v):
    assert len(nl) == len(ij)
    np.testing.assert_array_equal(nl[:], ij)
    np.testing.assert_array_equal(nl.distances, d)
    np.testing.assert_array_equal(nl.vectors, v)


@pytest.mark.parametrize("name", golden_names("ball_"))
def test_ball_golden(freud, name):
    g = load_golden(name)
    box = box_of(freud, g["box"])
    nq = make_nq(freud, int(g["kind"]), box, g["points"], float(g.get("cell_width", 0.0)))
    qp = g.get("query_points")
    args = dict(mode="ball", r_max=float(g["r_max"]), r_min=float(g.get("r_min", 0.0)), exclude_ii=qp is None)
    nl = nq.query(g["points"] if qp is None else qp, args).toNeighborList(sort_by_distance=name.endswith("_bydist"))
    assert_nlist_equal(nl, g["ij"], g["d"], g["v"])


@pytest.mark.parametrize("name", golden_names("knn_"))
def test_knn_golden(freud, name):
    g = load_golden(name)
    box = box_of(freud, g["box"])
    nq = make_nq(freud, int(g["kind"]), box, g["points"], 1.6)
    args = dict(num_neighbors=int(g["k"]), exclude_ii=name != "knn_aabb_rmax")
    if "r_max" in g:
        args["r_max"] = float(g["r_max"])
    nl = nq.query(g["points"], args).toNeighborList()
    assert_nlist_equal(nl, g["ij"], g["d"], g["v"])


def test_rdf_plain_golden(freud):
    g = load_golden("rdf_plain")
    rdf = freud.density.RDF(int(g["bins"]), float(g["r_max"]))
    rdf.compute((box_of(freud, g["box"]), g["points"]))
    np.testing.assert_array_equal(rdf.bin_counts, g["counts"])
    np.testing.assert_array_equal(rdf.rdf, g["rdf"])
    np.testing.assert_array_equal(rdf.n_r, g["n_r"])


def test_rdf_frames_golden(freud):
    g = load_golden("rdf_frames")
    rdf = freud.density.RDF(int(g["bins"]), float(g["r_max"]), float(g["r_min"]))
    for f in range(int(g["nframes"])):
        rdf.compute((box_of(freud, g["box%d" % f]), g["points%d" % f]), reset=(f == 0))
    np.testing.assert_array_equal(rdf.bin_counts, g["counts"])
    np.testing.assert_array_equal(rdf.rdf, g["rdf"])
    np.testing.assert_array_equal(rdf.n_r, g["n_r"])


def test_rdf_finite_size_golden(freud):
    g = load_golden("rdf_finite_size")
    rdf = freud.density.RDF(int(g["bins"]), float(g["r_max"]), normalization_mode="finite_size")
    rdf.compute((box_of(freud, g["box"]), g["points"]), neighbors={"r_max": float(g["r_max"]), "exclude_ii": False})
    np.testing.assert_array_equal(rdf.bin_counts, g["counts"])
    np.testing.assert_array_equal(rdf.rdf, g["rdf"])
    np.testing.assert_array_equal(rdf.n_r, g["n_r"])


@pytest.mark.parametrize("name", golden_names("st_"))
def test_steinhardt_golden(freud, name):
    g = load_golden(name)
    ls = [int(x) for x in g["ls"]]
    av, wl, wn = bool(g.get("average", 0)), bool(g.get("wl", 0)), bool(g.get("wl_normalize", 0))
    st = freud.order.Steinhardt(ls if len(ls) > 1 else ls[0], average=av, wl=wl, wl_normalize=wn)
    neighbors = {"r_max": float(g["r_max"])} if "r_max" in g else {"num_neighbors": 12}
    st.compute((box_of(freud, g["box"]), g["points"]), neighbors=neighbors)
    ql = np.atleast_2d(np.asarray(st.ql).T).T.reshape(g["ql"].shape)
    # Ql: 1e-5 relative to the reference (whose Ylm comes from the fsph stand-in)
    np.testing.assert_allclose(ql, g["ql"], rtol=1e-5, atol=1e-6)
    po = np.asarray(st.particle_order).reshape(g["particle_order"].shape)
    scale = np.max(np.abs(g["particle_order"]), axis=0)
    # Wl: the reference's own float32 triple sums sit up to 5.6e-6 of the |w| scale
    # from FP64 (W10); the values here are within 1e-5 |w| + 1e-7 of FP64
    assert np.all(np.abs(po - g["particle_order"]) <= 2e-5 * scale + 1e-7)
    np.testing.assert_allclose(np.atleast_1d(st.order), g["order"], rtol=5e-5, atol=1e-6)
    qlm = st.particle_harmonics
    qlm = np.concatenate([q.reshape(-1) for q in qlm]) if isinstance(qlm, list) else qlm.reshape(-1)
    np.testing.assert_allclose(qlm, g["qlm"], atol=5e-6)


# ---- larger seeded systems against the oracle ---------------------------------------

def random_box_points(freud, L, n, seed, tilt=(0, 0, 0), is2d=False):
    box = freud.box.Box(L, L, 0 if is2d else L, tilt[0], 0 if is2d else tilt[1], 0 if is2d else tilt[2], is2d)
    rs = np.random.RandomState(seed)
    f = rs.random_sample((n, 3))
    if is2d:
        f[:, 2] = 0
    return box, box.make_absolute(f)


@pytest.mark.parametrize("kind", [0, 2, 3])
@pytest.mark.parametrize("tilt", [(0, 0, 0), (0.2, 0.1, 0.0), (-0.4, 0.3, 0.2)])
def test_ball_vs_oracle_medium(freud, kind, tilt):
    box, pts = random_box_points(freud, 24.0, 20000, 7, tilt)
    nq = make_nq(freud, kind, box, pts, 3.0)
    nl = nq.query(pts, dict(r_max=3.0, exclude_ii=True)).toNeighborList()
    ij, d, v = O.query(box, pts, r_max=3.0, exclude_ii=True, arith=ARITH[kind])
    assert_nlist_equal(nl, ij, d, v)


@pytest.mark.parametrize("kind", [1, 2])
def test_knn_vs_oracle_medium(freud, kind):
    box, pts = random_box_points(freud, 20.0, 8000, 9, (0.1, 0.0, 0.05))
    nq = make_nq(freud, kind, box, pts, 2.0)
    for k in (1, 6, 12, 32):
        nl = nq.query(pts, dict(num_neighbors=k, exclude_ii=True)).toNeighborList()
        ij, d, v = O.query(box, pts, num_neighbors=k, exclude_ii=True, arith=ARITH[kind])
        assert_nlist_equal(nl, ij, d, v)


def test_knn_large_k_small_system(freud):
    box, pts = random_box_points(freud, 10.0, 500, 3)
    nq = freud.locality.AABBQuery(box, pts)
    nl = nq.query(pts, dict(num_neighbors=50, exclude_ii=True)).toNeighborList()
    ij, d, v = O.query(box, pts, num_neighbors=50, exclude_ii=True)
    assert_nlist_equal(nl, ij, d, v)


@pytest.mark.parametrize("kind", [1, 2])
def test_knn_large_k_many_points(freud, kind):
    """k > 32 on 12,000 points: the block brute force streams more accepted points
    than its 8,192-key buffer holds, cutting it to the k best as it fills."""
    box, pts = random_box_points(freud, 24.0, 12000, 21, (0.1, 0.0, 0.05))
    nq = make_nq(freud, kind, box, pts, 2.0)
    for k, r_max in ((40, None), (300, None), (64, 5.0)):
        args = dict(num_neighbors=k, exclude_ii=True)
        oargs = dict(num_neighbors=k, exclude_ii=True, arith=ARITH[kind])
        if r_max is not None:
            args["r_max"] = oargs["r_max"] = r_max
        nl = nq.query(pts, args).toNeighborList()
        ij, d, v = O.query(box, pts, **oargs)
        assert_nlist_equal(nl, ij, d, v)


def test_rdf_fused_vs_oracle_medium(freud):
    box, pts = random_box_points(freud, 21.544, 10000, 5)
    rdf = freud.density.RDF(200, 4.0)
    rdf.compute((box, pts))
    c = O.rdf_counts_query(box, pts, 200, 4.0)
    np.testing.assert_array_equal(rdf.bin_counts_u64, c)


def test_rdf_from_nlist_equals_fused(freud):
    box, pts = random_box_points(freud, 18.0, 6000, 6, (0.2, 0.0, 0.0))
    lc = freud.locality.LinkCell(box, pts, 3.0)
    nl = lc.query(pts, dict(r_max=3.0, exclude_ii=True)).toNeighborList()
    a = freud.density.RDF(300, 3.0).compute((box, pts), neighbors=nl)
    b = freud.density.RDF(300, 3.0).compute(lc, neighbors=dict(r_max=3.0))
    np.testing.assert_array_equal(a.bin_counts, b.bin_counts)
    c = O.hist(nl.distances, 300, 3.0)
    np.testing.assert_array_equal(a.bin_counts_u64, c)


def test_heavy_queries(freud):
    # dense system: every query has more bonds than the warp staging capacity
    box, pts = random_box_points(freud, 6.0, 4000, 8)
    for kind in (0, 2):
        nq = make_nq(freud, kind, box, pts, 2.9)
        nl = nq.query(pts, dict(r_max=2.9, exclude_ii=True)).toNeighborList()
        ij, d, v = O.query(box, pts, r_max=2.9, exclude_ii=True, arith=ARITH[kind])
        assert nl.neighbor_counts.max() > 256
        assert_nlist_equal(nl, ij, d, v)


@pytest.mark.parametrize("kind", [0, 2, 3])
@pytest.mark.parametrize("tilt", [(0, 0, 0), (0.2, 0.1, 0.0)])
def test_dense_ball_nlist(freud, kind, tilt):
    """Density 1 with r_max 4 (~2,000 candidates per 27-cell stencil): the
    block-per-cell kernels with a 4,096-candidate capacity."""
    box, pts = random_box_points(freud, 21.544, 10000, 12, tilt)
    nq = make_nq(freud, kind, box, pts, 4.0)
    nl = nq.query(pts, dict(r_max=4.0, exclude_ii=True)).toNeighborList()
    ij, d, v = O.query(box, pts, r_max=4.0, exclude_ii=True, arith=ARITH[kind])
    assert_nlist_equal(nl, ij, d, v)
    _, qpts = random_box_points(freud, 21.544, 3000, 13, tilt)
    nl = nq.query(qpts, dict(r_max=4.0, r_min=0.7)).toNeighborList()
    ij, d, v = O.query(box, pts, query_points=qpts, r_max=4.0, r_min=0.7, arith=ARITH[kind])
    assert_nlist_equal(nl, ij, d, v)


def test_dense_ball_nlist_with_overflow_cluster(freud):
    """Dense uniform points (4,096-candidate capacity) plus a tight cluster whose
    stencils exceed even that: those cells go to the warp-per-query kernels."""
    box, pts = random_box_points(freud, 21.544, 12000, 17)
    rs = np.random.RandomState(18)
    cluster = (rs.normal(0, 0.8, (3500, 3)) + np.array([2.0, -3.0, 1.0])).astype(np.float32)
    pts = np.concatenate([pts, cluster]).astype(np.float32)
    for kind in (0, 2):
        nq = make_nq(freud, kind, box, pts, 4.0)
        nl = nq.query(pts, dict(r_max=4.0, exclude_ii=True)).toNeighborList()
        ij, d, v = O.query(box, pts, r_max=4.0, exclude_ii=True, arith=ARITH[kind])
        assert nl.neighbor_counts.max() > 3000
        assert_nlist_equal(nl, ij, d, v)


@pytest.mark.parametrize("kind", [0, 2, 3])
def test_ball_queries_beyond_shared_capacity(freud, kind):
    """Query points inside a 12,000-point cluster: each has more bonds than the
    8,192-bond shared-memory staging of the heavy-query kernel, so its bonds are
    sorted in place in the output."""
    box, pts = random_box_points(freud, 20.0, 3000, 31)
    rs = np.random.RandomState(32)
    cluster = (rs.normal(0, 0.5, (12000, 3)) + np.array([1.0, 2.0, -1.5])).astype(np.float32)
    pts = np.concatenate([pts, cluster]).astype(np.float32)
    qpts = np.concatenate([cluster[:6], pts[:4]]).astype(np.float32)
    nq = make_nq(freud, kind, box, pts, 2.5)
    nl = nq.query(qpts, dict(r_max=2.5)).toNeighborList()
    ij, d, v = O.query(box, pts, query_points=qpts, r_max=2.5, arith=ARITH[kind])
    assert nl.neighbor_counts.max() > 9000
    assert_nlist_equal(nl, ij, d, v)


def test_dense_ball_nlist_2d(freud):
    box, pts = random_box_points(freud, 60.0, 20000, 14, (0.1, 0, 0), is2d=True)
    for kind in (0, 2):
        nq = make_nq(freud, kind, box, pts, 5.0)
        nl = nq.query(pts, dict(r_max=5.0, exclude_ii=True)).toNeighborList()
        ij, d, v = O.query(box, pts, r_max=5.0, exclude_ii=True, arith=ARITH[kind])
        assert_nlist_equal(nl, ij, d, v)


def test_dense_ball_nlist_wide_keys(freud):
    """More than 2^20 points with dense stencils: 64-bit merge keys at the
    4,096-candidate capacity. The first 2,000 queries' rows against the oracle."""
    box, pts = random_box_points(freud, 103.0, 1100000, 15)
    nq = freud.locality.LinkCell(box, pts, 4.0)
    nl = nq.query(pts, dict(r_max=4.0, exclude_ii=True)).toNeighborList()
    m = 2000
    ij, d, v = O.query(box, pts, query_points=pts[:m], r_max=4.0, exclude_ii=True, arith=O.ARITH_WRAP)
    nb = len(ij)
    np.testing.assert_array_equal(nl[:nb], ij)
    np.testing.assert_array_equal(nl.distances[:nb], d)
    np.testing.assert_array_equal(nl.vectors[:nb], v)
    assert nl[nb, 0] == m
    counts = nl.neighbor_counts
    assert counts.sum() == len(nl) and counts.min() > 150


def test_ball_nlist_wide_keys_sparse(freud):
    """More than 2^22 points at low density: 64-bit merge keys at the 1,024-candidate
    capacity. The first 3,000 queries' rows against the oracle."""
    box, pts = random_box_points(freud, 172.0, 4400000, 16, (0.1, 0.0, 0.0))
    nq = freud.locality.AABBQuery(box, pts)
    nl = nq.query(pts, dict(r_max=1.3, exclude_ii=True)).toNeighborList()
    m = 3000
    ij, d, v = O.query(box, pts, query_points=pts[:m], r_max=1.3, exclude_ii=True)
    nb = len(ij)
    np.testing.assert_array_equal(nl[:nb], ij)
    np.testing.assert_array_equal(nl.distances[:nb], d)
    np.testing.assert_array_equal(nl.vectors[:nb], v)
    assert nl[nb, 0] == m


def test_points_outside_box(freud):
    box, pts = random_box_points(freud, 10.0, 800, 4)
    shifted = pts.copy()
    shifted[::3] += np.float32(10.0)  # one box length: same wrapped system
    shifted[1::7] -= np.float32(10.0)
    for kind in (0, 2):
        nq = make_nq(freud, kind, box, shifted, 2.0)
        nl = nq.query(shifted, dict(r_max=2.0, exclude_ii=True)).toNeighborList()
        ij, d, v = O.query(box, shifted, r_max=2.0, exclude_ii=True, arith=ARITH[kind])
        assert_nlist_equal(nl, ij, d, v)


def test_small_box_few_cells(freud):
    # LinkCell radius close to half the box: one or two cells per dimension
    box, pts = random_box_points(freud, 5.0, 200, 12, (0.1, 0, 0))
    lc = freud.locality.LinkCell(box, pts, 2.4)
    nl = lc.query(pts, dict(r_max=2.45, exclude_ii=True)).toNeighborList()
    ij, d, v = O.query(box, pts, r_max=2.45, exclude_ii=True, arith=O.ARITH_WRAP)
    assert_nlist_equal(nl, ij, d, v)


def test_aabb_two_cells_per_axis(freud):
    # AABB arithmetic with two cells per axis: each cell appears twice in the
    # stencil (two images), so the candidate set holds every point twice
    box, pts = random_box_points(freud, 5.0, 300, 13, (0.1, 0.0, 0.0))
    nq = freud.locality.AABBQuery(box, pts)
    nl = nq.query(pts, dict(r_max=2.2, exclude_ii=True)).toNeighborList()
    ij, d, v = O.query(box, pts, r_max=2.2, exclude_ii=True, arith=O.ARITH_AABB)
    assert_nlist_equal(nl, ij, d, v)
    rdf = freud.density.RDF(50, 2.2).compute(nq, neighbors={"r_max": 2.2})
    np.testing.assert_array_equal(rdf.bin_counts_u64, O.hist(d, 50, 2.2))


def test_dense_blob_histogram(freud):
    # a dense blob: home cells with more candidates than the shared-memory tile
    rs = np.random.RandomState(21)
    box = freud.box.Box.cube(40.0)
    pts = np.concatenate([rs.normal(0, 1.5, (6000, 3)), rs.uniform(-20, 20, (4000, 3))]).astype(np.float32)
    pts = box.wrap(pts)
    rdf = freud.density.RDF(120, 3.0).compute((box, pts))
    np.testing.assert_array_equal(rdf.bin_counts_u64, O.rdf_counts_query(box, pts, 120, 3.0))
    lc = freud.locality.LinkCell(box, pts, 3.0)
    nl = lc.query(pts, dict(r_max=3.0, exclude_ii=True)).toNeighborList()
    ij, d, v = O.query(box, pts, r_max=3.0, exclude_ii=True, arith=O.ARITH_WRAP)
    assert_nlist_equal(nl, ij, d, v)
    rdf2 = freud.density.RDF(120, 3.0).compute(lc, neighbors={"r_max": 3.0})
    np.testing.assert_array_equal(rdf2.bin_counts_u64, O.hist(d, 120, 3.0))


@pytest.mark.parametrize("bins,r_max,r_min", [(200, 4.0, 0.0), (16, 4.0, 0.0), (500, 5.0, 0.0), (75, 3.75, 1.0),
                                              (1, 4.0, 0.0), (1000, 2.0, 0.5), (1500, 4.0, 0.0)])
def test_rdf_lattice_distances_on_bin_edges(freud, bins, r_max, r_min):
    """Simple-cubic lattice of spacing 0.5: every pair distance is the root of an
    integer multiple of 1/4, so many land exactly on bin edges (and on r_max): the
    r^2 -> bin tables must bin them as sqrt then truncation does. 1,500 bins
    exceed the table's capacity (square-root path)."""
    n = 22
    g = (np.arange(n, dtype=np.float32) - n / 2) * np.float32(0.5)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    box = freud.box.Box.cube(n * 0.5)
    rdf = freud.density.RDF(bins, r_max, r_min).compute((box, pts), neighbors={"r_max": r_max, "r_min": r_min,
                                                                               "exclude_ii": True})
    c = O.rdf_counts_query(box, pts, bins, r_max, r_min)
    np.testing.assert_array_equal(rdf.bin_counts_u64, c)
    assert c.sum() > 0


def test_empty_result(freud):
    box, pts = random_box_points(freud, 10.0, 100, 1)
    nq = freud.locality.AABBQuery(box, pts)
    nl = nq.query(pts, dict(r_max=1e-4, exclude_ii=True)).toNeighborList()
    assert len(nl) == 0
    assert nl[:].shape == (0, 2)
    np.testing.assert_array_equal(nl.neighbor_counts, np.zeros(100, np.uint32))


@pytest.mark.parametrize("average", [True, False])
def test_steinhardt_vs_fp64_oracle(freud, average):
    """16,384-point noisy FCC crystal, 12 nearest neighbours, l = 4..12: Ql within
    1e-5 relative of the FP64 oracle; normalised Wl within 1e-5 |w| + 1e-7 for every
    particle and l, W10 included (its Wigner-3j triple sum cancels hardest on FCC,
    so the Wl path computes the harmonics and the sums over bonds in float-float)."""
    from golden.make_golden import fcc

    box, pts = fcc(16, 1.5874, 0.05, 77)
    fbox = box_of(freud, np.asarray(box, np.float32))
    ls = [4, 6, 8, 10, 12]
    st = freud.order.Steinhardt(ls, average=average, wl=True, wl_normalize=True)
    st.compute((fbox, pts), neighbors={"num_neighbors": 12})
    ij, d, v = O.query(box, pts, num_neighbors=12, exclude_ii=True)
    o = O.steinhardt(ls, box, pts, ij, d, average=average, wl=True, wl_normalize=True)
    np.testing.assert_allclose(st.ql, o["ql_ave"] if average else o["ql"], rtol=1e-5)
    w = o["wl"]
    err = np.abs(st.particle_order - w)
    print("max |dw| / (1e-5 |w| + 1e-7) per l:", np.max(err / (1e-5 * np.abs(w) + 1e-7), axis=0))
    assert np.all(err <= 1e-5 * np.abs(w) + 1e-7)
    np.testing.assert_allclose(np.atleast_1d(st.order), o["order"], rtol=1e-5, atol=1e-7)
    st2 = freud.order.Steinhardt(ls)
    st2.compute((fbox, pts), neighbors={"num_neighbors": 12})
    o2 = O.steinhardt(ls, box, pts, ij, d)
    np.testing.assert_allclose(st2.ql, o2["ql"], rtol=1e-5)
    np.testing.assert_allclose(np.atleast_1d(st2.order), o2["order"], rtol=1e-5)


# ---- CellQuery (ghost copies; third pair arithmetic) -----------------------------------

def test_rdf_cellquery_golden(freud):
    g = load_golden("rdf_cellquery")
    box = box_of(freud, g["box"])
    rdf = freud.density.RDF(int(g["bins"]), float(g["r_max"]))
    rdf.compute(freud.locality.CellQuery(box, g["points"]))
    np.testing.assert_array_equal(rdf.bin_counts, g["counts"])
    np.testing.assert_array_equal(rdf.rdf, g["rdf"])
    np.testing.assert_array_equal(rdf.n_r, g["n_r"])


@pytest.mark.parametrize("spill", [0.0, 0.08])
def test_cellquery_points_outside_box(freud, spill):
    """Points up to 8% of the box outside it: their copies beyond the padded grid are
    dropped, as the reference drops them; query points partly outside the grid."""
    rs = np.random.RandomState(5)
    box = freud.box.Box(14.0, 13.0, 15.0, 0.3, -0.2, 0.1)
    pts = box.make_absolute(rs.random_sample((6000, 3)) * (1 + 2 * spill) - spill).astype(np.float32)
    qp = box.make_absolute(rs.random_sample((900, 3)) * 1.3 - 0.15).astype(np.float32)
    nq = freud.locality.CellQuery(box, pts)
    nl = nq.query(pts, dict(r_max=2.6, r_min=0.3, exclude_ii=True)).toNeighborList()
    assert_nlist_equal(nl, *O.query(box, pts, r_max=2.6, r_min=0.3, exclude_ii=True, arith=O.ARITH_GHOST))
    nl = nq.query(qp, dict(r_max=2.6)).toNeighborList(sort_by_distance=True)
    assert_nlist_equal(nl, *O.query(box, pts, query_points=qp, r_max=2.6, arith=O.ARITH_GHOST,
                                    sort_by_distance=True))
    counts = O.rdf_counts_query(box, pts, 100, 2.6, arith=O.ARITH_GHOST)
    rdf = freud.density.RDF(100, 2.6).compute(nq)
    np.testing.assert_array_equal(rdf.bin_counts_u64, counts)


def test_cellquery_dense_cells(freud):
    """Dense clusters (> 1024 candidates per cell) take the warp-per-query path."""
    rs = np.random.RandomState(8)
    box = freud.box.Box.cube(20.0)
    centres = rs.random_sample((6, 3)) * 20 - 10
    pts = (centres[:, None, :] + rs.normal(0, 0.6, (6, 700, 3))).reshape(-1, 3)
    pts = box.wrap(pts.astype(np.float32)).astype(np.float32)
    nq = freud.locality.CellQuery(box, pts)
    nl = nq.query(pts, dict(r_max=2.0, exclude_ii=True)).toNeighborList()
    assert_nlist_equal(nl, *O.query(box, pts, r_max=2.0, exclude_ii=True, arith=O.ARITH_GHOST))


def test_cellquery_errors(freud):
    box = freud.box.Box.cube(10.0)
    pts = np.zeros((4, 3), np.float32)
    nq = freud.locality.CellQuery(box, pts)
    with pytest.raises(RuntimeError, match="only supports ball queries"):
        nq.query(pts, dict(num_neighbors=2)).toNeighborList()
    with pytest.raises(RuntimeError, match="CellQuery r_max is too large"):
        nq.query(pts, dict(r_max=5.5)).toNeighborList()
    with pytest.raises(ValueError, match="r_max must be greater than r_min"):
        nq.query(pts, dict(r_max=1.0, r_min=2.0)).toNeighborList()


def test_box_division_matches_ieee(freud):
    """The box arithmetic divides by box lengths through a precomputed reciprocal
    with a Markstein correction; 2^30 seeded quotients (box lengths and random
    divisors, dividends of either sign over 24 binades) equal CUDA's IEEE division
    bit for bit."""
    import ctypes

    from freud_gb300 import _lib

    mism = ctypes.c_uint64()
    ex = (ctypes.c_float * 2)()
    _lib.check(_lib.lib.fg_check_division(1 << 30, 12345, ctypes.byref(mism), ex))
    assert mism.value == 0, "first differing (a, b) = (%r, %r)" % (ex[0], ex[1])
