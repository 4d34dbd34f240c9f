"""Fused RDF of (box, points) systems, where each unordered pair is counted once
from half of the stencil (pairs of image 0 tested once and counted twice, pairs
across the periodic boundary tested from both ends): bin counts against the
oracle's full double loop, bit for bit, over the cases that change which half
is taken."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def frame(freud, n, L, tilt=(0.0, 0.0, 0.0), is2d=False, seed=0, outside=False):
    box = freud.box.Box(L, L, 0.0 if is2d else L, tilt[0], 0.0 if is2d else tilt[1], 0.0 if is2d else tilt[2],
                        is2d)
    rs = np.random.RandomState(seed)
    f = rs.random_sample((n, 3))
    if is2d:
        f[:, 2] = 0
    pts = box.make_absolute(f).astype(np.float32)
    if outside:
        pts[::5] += np.float32(box.Lx)
    return box, pts


CASES = {
    "cubic": dict(n=6000, L=18.0),
    "triclinic": dict(n=6000, L=18.0, tilt=(0.5, 0.3, -0.2)),
    "2d": dict(n=5000, L=60.0, is2d=True),
    "2d_tilted": dict(n=5000, L=60.0, is2d=True, tilt=(0.3, 0.0, 0.0)),
    "few_cells": dict(n=400, L=5.2),
    "outside": dict(n=4000, L=16.0, outside=True),
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("r_min", [0.0, 0.7])
def test_single_frame_vs_oracle(freud, name, r_min):
    box, pts = frame(freud, seed=hash(name) % 1000, **CASES[name])
    r_max = 2.5
    rdf = freud.density.RDF(160, r_max, r_min).compute((box, pts))
    c = O.rdf_counts_query(box, pts, 160, r_max, r_min=r_min, arith=O.ARITH_AABB)
    np.testing.assert_array_equal(rdf.bin_counts_u64, c)


@pytest.mark.parametrize("config", [(1, 8, 1), (2, 4, 2)])
def test_frames_mixed_vs_oracle(freud, config):
    """A batch whose frames differ in shape, dimension of the cell grid and whether
    points lie outside the box (that frame keeps the whole stencil)."""
    frames = [frame(freud, seed=s, **kw) for s, kw in enumerate([
        dict(n=3000, L=15.0), dict(n=3000, L=15.0, tilt=(0.2, 0.1, 0.0)), dict(n=300, L=5.0),
        dict(n=2500, L=14.0, outside=True), dict(n=5000, L=17.5, tilt=(-0.4, 0.2, 0.3))])]
    counts = np.zeros(200, np.uint64)
    for box, pts in frames:
        O.rdf_counts_query(box, pts, 200, 2.2, arith=O.ARITH_AABB, counts=counts)
    freud._lib.set_batch_config(*config)
    try:
        rdf = freud.density.RDF(200, 2.2).compute(freud.locality.FrameBatch(frames))
    finally:
        freud._lib.set_batch_config(0)
    np.testing.assert_array_equal(rdf.bin_counts_u64, counts)


def test_dense_blobs_vs_oracle(freud):
    """Gaussian blobs: stencils above the 1,024-candidate tile (several tiles per
    cell) and bins whose counts go well above 2^16."""
    rs = np.random.RandomState(5)
    L = 40.0
    centres = rs.uniform(-L / 2, L / 2, (24, 3))
    pts = (centres[:, None, :] + rs.normal(0.0, 1.5, (24, 800, 3))).reshape(-1, 3)
    pts = ((pts + L / 2) % L - L / 2).astype(np.float32)
    box = freud.box.Box.cube(L)
    rdf = freud.density.RDF(300, 4.0).compute((box, pts))
    c = O.rdf_counts_query(box, pts, 300, 4.0, arith=O.ARITH_AABB)
    np.testing.assert_array_equal(rdf.bin_counts_u64, c)


def test_without_exclude_ii_vs_oracle(freud):
    """exclude_ii off: each point's pair with itself is counted in bin 0 (whole stencil)."""
    box, pts = frame(freud, 3000, 14.0, seed=9)
    rdf = freud.density.RDF(100, 2.0).compute((box, pts), neighbors={"r_max": 2.0, "exclude_ii": False})
    c = O.rdf_counts_query(box, pts, 100, 2.0, exclude_ii=False, arith=O.ARITH_AABB)
    np.testing.assert_array_equal(rdf.bin_counts_u64, c)
