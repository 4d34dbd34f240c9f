"""NeighborList build on the GPU: the lanes-over-queries count pass against the
block-per-cell one and against the oracle, bit for bit, including the jittered
simple-cubic lattice of the large-N workload at 48^3 points."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def lattice(n1, seed=2024, sigma=0.1):
    """n1^3 simple-cubic lattice of spacing 1 with N(0, sigma) jitter, wrapped into
    the periodic cube of side n1 (the large-N workload's generator)."""
    L = float(n1)
    g = np.arange(n1, dtype=np.float64) - n1 / 2.0
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
    rng = np.random.default_rng(seed)
    pts = pts + rng.normal(0.0, sigma, pts.shape)
    pts = (pts + L / 2) % L - L / 2
    return L, pts.astype(np.float32)


def lists_equal(a, b):
    return (len(a) == len(b) and np.array_equal(a[:], b[:]) and
            np.array_equal(a.distances.view(np.uint32), b.distances.view(np.uint32)) and
            np.array_equal(a.vectors.view(np.uint32), b.vectors.view(np.uint32)))


def assert_oracle(nl, ij, d, v):
    assert len(nl) == len(ij)
    np.testing.assert_array_equal(nl[:], ij)
    np.testing.assert_array_equal(nl.distances.view(np.uint32), d.view(np.uint32))
    np.testing.assert_array_equal(nl.vectors.view(np.uint32), v.view(np.uint32))


@pytest.fixture
def both_kernels(freud):
    from freud_gb300 import _lib

    def run(fn):
        out = []
        for which in (0, 1):
            _lib.set_count_kernel(which)
            try:
                out.append(fn())
            finally:
                _lib.set_count_kernel(0)
        return out

    return run


def test_lattice_48_vs_oracle(freud):
    """The large-N workload's lattice at 48^3 = 110,592 points (LinkCell w = 3,
    r_max = 3): the whole list and its RDF(300, 3.0) counts equal the oracle's."""
    L, pts = lattice(48)
    box = freud.box.Box.cube(L)
    lc = freud.locality.LinkCell(box, pts, 3.0)
    nl = lc.query(pts, {"r_max": 3.0, "exclude_ii": True}).toNeighborList()
    ij, d, v = O.query((L, L, L, 0.0, 0.0, 0.0, 0.0), pts, r_max=3.0, exclude_ii=True, arith=O.ARITH_WRAP)
    assert_oracle(nl, ij, d, v)
    rdf = freud.density.RDF(300, 3.0).compute(lc, neighbors=nl)
    np.testing.assert_array_equal(rdf.bin_counts_u64, O.hist(d, 300, 3.0))


@pytest.mark.parametrize("case", ["cubic", "triclinic", "2d", "rmin", "query_points", "outside", "jitter"])
def test_count_kernels_agree(freud, both_kernels, case):
    rs = np.random.RandomState(41)
    tilt, is2d, L, n, r, rmin = (0.0, 0.0, 0.0), False, 24.0, 20000, 3.0, 0.0
    if case == "triclinic":
        tilt = (0.3, -0.2, 0.1)
    if case == "2d":
        is2d, L, n = True, 80.0, 20000
    if case == "rmin":
        rmin = 1.1
    box = freud.box.Box(L, L, 0 if is2d else L, tilt[0], 0 if is2d else tilt[1], 0 if is2d else tilt[2], is2d)
    f = rs.random_sample((n, 3))
    if is2d:
        f[:, 2] = 0
    pts = box.make_absolute(f).astype(np.float32)
    if case == "jitter":
        L, pts = lattice(30, seed=5, sigma=0.3)
        box = freud.box.Box.cube(L)
    if case == "outside":
        pts[::3] += np.float32(L)
        pts[1::7] -= np.float32(L)
    qpts = pts
    args = {"r_max": r, "r_min": rmin, "exclude_ii": True}
    if case == "query_points":
        qf = rs.random_sample((5000, 3))
        qpts = box.make_absolute(qf).astype(np.float32)
        qpts[:100] = pts[:100]  # some query points on points: exclude_ii by index
    lc = freud.locality.LinkCell(box, pts, r)
    new, old = both_kernels(lambda: lc.query(qpts, args).toNeighborList())
    assert lists_equal(new, old)
    ij, d, v = O.query(box, pts, query_points=None if qpts is pts else qpts, r_max=r, r_min=rmin,
                       exclude_ii=True, arith=O.ARITH_WRAP)
    assert_oracle(new, ij, d, v)


def test_count_kernel_wide_keys(freud, both_kernels):
    """More than 2^22 points (64-bit merge keys) at LinkCell arithmetic; the first
    3,000 queries' rows against the oracle and both count kernels equal."""
    rs = np.random.RandomState(43)
    box = freud.box.Box(172.0, 172.0, 172.0, 0.1, 0.0, 0.0)
    pts = box.make_absolute(rs.random_sample((4400000, 3))).astype(np.float32)
    lc = freud.locality.LinkCell(box, pts, 1.3)
    new, old = both_kernels(lambda: lc.query(pts, {"r_max": 1.3, "exclude_ii": True}).toNeighborList())
    assert lists_equal(new, old)
    m = 3000
    ij, d, v = O.query(box, pts, query_points=pts[:m], r_max=1.3, exclude_ii=True, arith=O.ARITH_WRAP)
    nb = len(ij)
    np.testing.assert_array_equal(new[:nb], ij)
    np.testing.assert_array_equal(new.distances[:nb], d)
    np.testing.assert_array_equal(new.vectors[:nb], v)
    assert new[nb, 0] == m


def test_count_kernel_dense_cluster(freud, both_kernels):
    """Uniform points plus a tight cluster: cells whose culled stencils exceed
    1,024 candidates go to the warp-per-query kernels from either count pass."""
    rs = np.random.RandomState(44)
    box = freud.box.Box.cube(30.0)
    pts = box.make_absolute(rs.random_sample((20000, 3))).astype(np.float32)
    cluster = (rs.normal(0, 0.6, (2500, 3)) + np.array([3.0, -2.0, 1.0])).astype(np.float32)
    pts = np.concatenate([pts, cluster]).astype(np.float32)
    lc = freud.locality.LinkCell(box, pts, 2.5)
    new, old = both_kernels(lambda: lc.query(pts, {"r_max": 2.5, "exclude_ii": True}).toNeighborList())
    assert lists_equal(new, old)
    ij, d, v = O.query(box, pts, r_max=2.5, exclude_ii=True, arith=O.ARITH_WRAP)
    assert_oracle(new, ij, d, v)


def test_large_list_readback_in_page_locked_arrays(freud):
    """A list of at least 2^20 bonds comes back in pooled page-locked arrays: read-only,
    bit-equal to the oracle's list, and a dropped list's blocks return to the pool."""
    import gc

    from freud_gb300 import _lib

    rs = np.random.RandomState(47)
    box = freud.box.Box.cube(40.0)
    pts = box.make_absolute(rs.random_sample((60000, 3))).astype(np.float32)
    nl = freud.locality.LinkCell(box, pts, 2.5).query(pts, {"r_max": 2.5, "exclude_ii": True}).toNeighborList()
    assert len(nl) >= 1 << 20
    ij, d, v = nl[:], nl.distances, nl.vectors
    for a in (ij, d, v):
        assert not a.flags.writeable
    oij, od, ov = O.query(O.box7(box), pts, r_max=2.5, exclude_ii=True, arith=O.ARITH_WRAP)
    np.testing.assert_array_equal(ij, oij)
    np.testing.assert_array_equal(d, od)
    np.testing.assert_array_equal(v, ov)
    pooled = sum(len(x) for x in _lib._pinned_free.values())
    del ij, d, v, nl, a
    gc.collect()
    assert sum(len(x) for x in _lib._pinned_free.values()) >= pooled + 3
