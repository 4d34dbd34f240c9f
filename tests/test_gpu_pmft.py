"""PMFTs on the GPU against the reference's fixtures (tests/golden/pmft_*.npz,
from PMFTR12.cc / PMFTXYT.cc / PMFTXY.cc / PMFTXYZ.cc) and the reference's own
test cases (tests/test_pmft.py). XYZ bins are pure float arithmetic: counts and
pcf equal. R12 and XYT take atan2 on the device and XY / XYT the rotation's
cos / sin from the host C library, so a bond within an ulp of a bin edge may land
in the neighbouring bin: counts may differ by at most 1e-4 of the bonds (and
the pcf with them); in practice they are equal."""

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _box(freud, b):
    return freud.box.Box(float(b[0]), float(b[1]), float(b[2]), float(b[3]), float(b[4]), float(b[5]), bool(b[6]))


def _close_counts(got, want):
    moved = int(np.abs(got.astype(np.int64) - want.astype(np.int64)).sum())
    assert moved <= max(2, int(1e-4 * want.sum())), moved
    return moved


def test_pmft_r12_golden(freud):
    g = load_golden("pmft_r12")
    pm = freud.pmft.PMFTR12(3.0, tuple(int(b) for b in g["bins"]))
    for f in range(int(g["nframes"])):
        pm.compute((_box(freud, g["box%d" % f]), g["points%d" % f]), g["orient%d" % f], reset=False)
    if _close_counts(pm.bin_counts, g["counts"]) == 0:
        np.testing.assert_array_equal(pm._pcf, g["pcf"])
    assert pm.box == _box(freud, g["box1"])


def test_pmft_xyt_xy_golden(freud):
    g = load_golden("pmft_xyt")
    pm = freud.pmft.PMFTXYT(3.0, 2.5, tuple(int(b) for b in g["bins"]))
    pm.compute((_box(freud, g["box0"]), g["points0"]), g["orient0"])
    if _close_counts(pm.bin_counts, g["counts"]) == 0:
        np.testing.assert_array_equal(pm._pcf, g["pcf"])
    g = load_golden("pmft_xy")
    pm = freud.pmft.PMFTXY(3.0, 3.0, tuple(int(b) for b in g["bins"]))
    pm.compute((_box(freud, g["box0"]), g["points0"]), g["query_orient"], query_points=g["query_points"])
    if _close_counts(pm.bin_counts, g["counts"]) == 0:
        np.testing.assert_array_equal(pm._pcf, g["pcf"])


def test_pmft_xyz_golden(freud):
    g = load_golden("pmft_xyz")
    pm = freud.pmft.PMFTXYZ(2.5, 2.5, 2.5, 10, shiftvec=g["shiftvec"].tolist())
    pm.compute((_box(freud, g["box0"]), g["points0"]), g["query_quats"], equiv_orientations=g["equiv"])
    np.testing.assert_array_equal(pm.bin_counts, g["counts"])
    np.testing.assert_array_equal(pm._pcf, g["pcf"])
    with np.errstate(divide="ignore"):
        np.testing.assert_array_equal(pm.pmft, -np.log(g["pcf"]))
    with pytest.raises(RuntimeError):
        pm.compute((_box(freud, g["box0"]), g["points0"]), g["query_quats"], equiv_orientations=g["equiv"][:1],
                   reset=False)


def test_pmft_nlist_equals_live(freud):
    g = load_golden("pmft_xyt")
    box = _box(freud, g["box0"])
    nq = freud.locality.AABBQuery(box, g["points0"])
    nl = nq.query(g["points0"], dict(r_max=float(g["r_max"]), exclude_ii=True)).toNeighborList()
    a = freud.pmft.PMFTXYT(3.0, 2.5, (12, 10, 6)).compute(nq, g["orient0"], neighbors=nl)
    b = freud.pmft.PMFTXYT(3.0, 2.5, (12, 10, 6)).compute(nq, g["orient0"])
    np.testing.assert_array_equal(a.bin_counts, b.bin_counts)


@pytest.mark.parametrize("which", ["R12", "XYT", "XY", "XYZ"])
def test_pmft_reference_behaviour(freud, which):
    """tests/test_pmft.py: box dimensionality, attribute access, shapes, repr, bins."""
    mk = {"R12": lambda: freud.pmft.PMFTR12(5.23, (10, 8, 6)),
          "XYT": lambda: freud.pmft.PMFTXYT(3.6, 4.2, (20, 30, 40)),
          "XY": lambda: freud.pmft.PMFTXY(3.6, 4.2, (20, 30)),
          "XYZ": lambda: freud.pmft.PMFTXYZ(5.23, 6.23, 7.23, (20, 30, 40))}[which]
    pm = mk()
    ndim = 3 if which == "XYZ" else 2
    L = 25 if ndim == 3 else 16
    box = freud.box.Box.cube(L) if ndim == 3 else freud.box.Box.square(L)
    other = freud.box.Box.square(L) if ndim == 3 else freud.box.Box.cube(L)
    points = np.array([[-1.0, 0.0, 0.0], [1.0, 0.1, 0.0]], dtype=np.float32)
    orientations = np.array([[1, 0, 0, 0], [1, 0, 0, 0]], dtype=np.float32)
    for attr in ("bin_counts", "box", "pmft"):
        with pytest.raises(AttributeError):
            getattr(pm, attr)
    pm.compute((box, points), orientations, reset=False)
    assert pm.bin_counts.shape == tuple(pm.nbins) and pm.pmft.shape == tuple(pm.nbins)
    assert pm.box == box
    assert pm.bin_counts.sum() == 2
    with pytest.raises(ValueError, match="only supports"):
        pm.compute((other, points), orientations)
    assert str(pm) == str(eval(repr(pm), {"freud": freud, "np": np}))
    for e, c, n in zip(pm.bin_edges, pm.bin_centers, pm.nbins):
        assert len(e) == n + 1 and len(c) == n
        np.testing.assert_allclose(c, (e[1:] + e[:-1]) / 2, atol=1e-6)
    if ndim == 2:
        # angles and z-rotation quaternions give the same counts
        ang = np.array([0.3, 1.2], np.float32)
        quat = np.stack([np.cos(ang / 2), 0 * ang, 0 * ang, np.sin(ang / 2)], 1)
        a = mk().compute((box, points), ang).bin_counts
        b = mk().compute((box, points), quat).bin_counts
        np.testing.assert_array_equal(a, b)
        with pytest.raises(ValueError):
            mk().compute((box, points), np.array([[0.9, 0.3, 0.0, 0.3], [1, 0, 0, 0]]))


def test_pmft_large_vs_oracle(freud):
    """20 k points in 2D, XYT with 40^3 bins: the oracle's counts within the atan2 tolerance."""
    from oracle import oracle as O

    rs = np.random.RandomState(120)
    L = 140.0
    box = freud.box.Box.square(L)
    pts = np.zeros((20000, 3), np.float32)
    pts[:, :2] = ((rs.random_sample((20000, 2)) - 0.5) * L).astype(np.float32)
    o = (rs.random_sample(20000) * 2 * np.pi).astype(np.float32)
    pm = freud.pmft.PMFTXYT(3.0, 3.0, 40).compute((box, pts), o)
    rm = float(np.float32(np.sqrt(18.0)))
    b = (L, L, 0.0, 0.0, 0.0, 0.0, 1)
    ij, d, v = O.query(b, pts, r_max=rm, exclude_ii=True)
    want = O.pmft_counts(1, [3.0, 3.0], [40, 40, 40], ij, d, v, p_angle=o, q_angle=o)
    _close_counts(pm.bin_counts, want)
