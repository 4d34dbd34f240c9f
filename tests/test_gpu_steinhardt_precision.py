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
