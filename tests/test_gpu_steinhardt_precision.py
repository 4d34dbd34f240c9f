"""Steinhardt accuracy against the FP64 oracle where float32 harmonics are most
fragile: bonds close to the z axis (sin(theta) from 1 - cos^2 cancels) and
averaged Ql of disordered frames (the neighbour average cancels). Ql within
1e-5 relative of the oracle for every particle."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel_err(got, ref):
    ok = np.isfinite(ref)
    assert np.array_equal(np.isfinite(got), ok)
    return float(np.max(np.abs(got[ok] - ref[ok]) / np.abs(ref[ok])))


def test_near_polar_bonds(freud):
    """Simple-cubic lattice with 0.01 jitter: the +-z bonds of every point sit
    within ~0.01 rad of the poles."""
    n1 = 24
    g = np.arange(n1, dtype=np.float64) - n1 / 2.0
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(7)
    pts = (pts + rng.normal(0, 0.01, pts.shape)).astype(np.float32)
    box = freud.box.Box.cube(float(n1))
    for ls, avg in (([4, 6, 8], False), ([6], True)):
        st = freud.order.Steinhardt(ls, average=avg)
        st.compute((box, pts), neighbors={"num_neighbors": 6})
        ij, d, _ = O.query(box, pts, num_neighbors=6, exclude_ii=True)
        o = O.steinhardt(ls, box, pts, ij, d, average=avg)
        ref = o["ql_ave"] if avg else o["ql"]
        got = np.asarray(st.ql, np.float64).reshape(ref.shape)
        assert rel_err(got, ref) <= 1e-5


@pytest.mark.parametrize("tilt", [(0.0, 0.0, 0.0), (0.2, 0.1, 0.0)])
def test_disordered_averaged_q6(freud, tilt):
    """120,000 uniform points at density 0.85 (the uneven trajectory's frames):
    Steinhardt(6, average) on r_max 1.5 ball neighbours."""
    n = 120000
    L = float((n / 0.85) ** (1.0 / 3.0))
    box = freud.box.Box(L, L, L, *tilt)
    rng = np.random.default_rng(11)
    pts = box.make_absolute(rng.random((n, 3))).astype(np.float32)
    st = freud.order.Steinhardt(6, average=True)
    st.compute((box, pts), neighbors={"r_max": 1.5})
    bx = O.box7(box)
    ij, d, _ = O.query(bx, pts, r_max=1.5, exclude_ii=True)
    o = O.steinhardt([6], bx, pts, ij, d, average=True)
    assert rel_err(np.asarray(st.ql, np.float64), o["ql_ave"][:, 0]) <= 1e-5


WL_FLOOR = 1e-7


def wl_check(got, ref):
    ok = np.isfinite(ref)
    assert np.array_equal(np.isfinite(got), ok)
    err = np.abs(got[ok] - ref[ok])
    assert np.all(err <= 1e-5 * np.abs(ref[ok]) + WL_FLOOR), float(np.max(err / (1e-5 * np.abs(ref[ok]) + WL_FLOOR)))


@pytest.mark.parametrize("tilt", [(0.0, 0.0, 0.0), (0.2, 0.1, 0.0)])
def test_wl_ball_neighbours(freud, tilt):
    """Normalised W4, W6, W10 (unaveraged) of a noisy FCC crystal in a cubic and a
    tilted box on r_max = 1.4 ball neighbours (uneven bond counts, odd ones
    included): within 1e-5 |w| + 1e-7 of the FP64 oracle."""
    from golden.make_golden import fcc

    box, pts = fcc(12, 1.5874, 0.08, 5)
    L = box[0]
    fbox = freud.box.Box(L, L, L, *tilt)
    pts = np.asarray(fbox.wrap(pts), np.float32)
    ls = [4, 6, 10]
    st = freud.order.Steinhardt(ls, wl=True, wl_normalize=True)
    st.compute((fbox, pts), neighbors={"r_max": 1.4})
    bx = O.box7(fbox)
    ij, d, _ = O.query(bx, pts, r_max=1.4, exclude_ii=True)
    counts = np.bincount(ij[:, 0], minlength=len(pts))
    assert np.any(counts % 2 == 1)
    o = O.steinhardt(ls, bx, pts, ij, d, wl=True, wl_normalize=True)
    np.testing.assert_allclose(np.asarray(st.ql, np.float64), o["ql"], rtol=1e-5)
    wl_check(np.asarray(st.particle_order, np.float64), o["wl"])


def test_wl_batched_frames(freud):
    """Wl through a FrameBatch (bond vectors precomputed per frame): two noisy FCC
    frames of different sizes, Steinhardt([6, 10], average, wl) on r_max 1.4."""
    from golden.make_golden import fcc

    frames = []
    for nc, seed in ((8, 1), (11, 2)):
        box, pts = fcc(nc, 1.5874, 0.06, seed)
        frames.append((freud.box.Box.cube(float(box[0])), pts))
    st = freud.order.Steinhardt([6, 10], average=True, wl=True, wl_normalize=True)
    st.compute(freud.locality.FrameBatch(frames), neighbors={"r_max": 1.4})
    got = np.asarray(st.particle_order, np.float64).reshape(-1, 2)
    start = 0
    for fbox, pts in frames:
        bx = O.box7(fbox)
        ij, d, _ = O.query(bx, pts, r_max=1.4, exclude_ii=True)
        o = O.steinhardt([6, 10], bx, pts, ij, d, average=True, wl=True, wl_normalize=True)
        wl_check(got[start:start + len(pts)], o["wl"])
        start += len(pts)
