"""Batched frames on the GPU: FrameBatch computes against the per-frame path and
the oracle. RDF counts (and the float32 rdf / n_r) must be bit-identical to one
compute(reset=False) per frame; Steinhardt per frame within the FP64-oracle
tolerances of the per-frame tests."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def make_frames(freud, sizes, seed, density=0.85, tilt_every=3, is2d=False, unwrapped=False):
    """Uniform points in fractional coordinates; every tilt_every-th box triclinic."""
    rs = np.random.RandomState(seed)
    frames = []
    for f, n in enumerate(sizes):
        if is2d:
            L = float((n / density) ** 0.5)
            box = freud.box.Box.square(L)
        else:
            L = float((n / density) ** (1.0 / 3.0))
            tilt = (0.2, 0.1, 0.0) if tilt_every and f % tilt_every == tilt_every - 1 else (0.0, 0.0, 0.0)
            box = freud.box.Box(L, L, L, *tilt)
        frac = rs.random_sample((n, 3))
        if is2d:
            frac[:, 2] = 0
        pts = box.make_absolute(frac).astype(np.float32)
        if unwrapped:
            # whole box lengths added to some points: same physics, images != 0
            shift = rs.randint(-1, 2, size=(n, 1)).astype(np.float32)
            pts = (pts + shift * np.array([box.Lx, 0.0, 0.0], np.float32)).astype(np.float32)
        frames.append((box, pts))
    return frames


def per_frame_rdf(freud, frames, bins, r_max, r_min=0.0):
    rdf = freud.density.RDF(bins, r_max, r_min)
    for f, (box, pts) in enumerate(frames):
        rdf.compute((box, pts), reset=(f == 0))
    return rdf


SIZES = [1200, 180, 4000, 800, 2500, 150, 3333]


@pytest.mark.parametrize("config", [(0, 8, 1), (1, 4, 1), (1, 8, 2), (2, 4, 2), (2, 8, 1)])
def test_rdf_frames_equal_per_frame(freud, config):
    frames = make_frames(freud, SIZES, 11)
    ref = per_frame_rdf(freud, frames, 200, 2.5)
    # oracle: sum of per-frame AABB-arithmetic counts
    counts = np.zeros(200, np.uint64)
    for box, pts in frames:
        O.rdf_counts_query(box, pts, 200, 2.5, arith=O.ARITH_AABB, counts=counts)
    freud._lib.set_batch_config(*config)
    try:
        rdf = freud.density.RDF(200, 2.5)
        rdf.compute(freud.locality.FrameBatch(frames), reset=False)
    finally:
        freud._lib.set_batch_config(0)
    np.testing.assert_array_equal(rdf.bin_counts_u64, counts)
    np.testing.assert_array_equal(rdf.bin_counts, ref.bin_counts)
    np.testing.assert_array_equal(rdf.rdf, ref.rdf)
    np.testing.assert_array_equal(rdf.n_r, ref.n_r)
    b, rb = rdf.box, ref.box
    assert (b.Lx, b.Ly, b.Lz, b.xy, b.xz, b.yz) == (rb.Lx, rb.Ly, rb.Lz, rb.xy, rb.xz, rb.yz)


def test_rdf_frames_autotuned_then_replayed(freud):
    """The first call tunes the launch shape; later calls replay the recorded graph.
    reset=False keeps adding: two calls give twice the counts."""
    frames = make_frames(freud, [3000, 700, 2200], 5)
    batch = freud.locality.FrameBatch(frames)
    rdf = freud.density.RDF(150, 3.0, 0.5)
    rdf.compute(batch, reset=False)
    once = rdf.bin_counts_u64.copy()
    rdf.compute(batch, reset=False)
    np.testing.assert_array_equal(rdf.bin_counts_u64, 2 * once)
    counts = np.zeros(150, np.uint64)
    for box, pts in frames:
        O.rdf_counts_query(box, pts, 150, 3.0, r_min=0.5, arith=O.ARITH_AABB, counts=counts)
    np.testing.assert_array_equal(once, counts)
    assert "rdf_frames" in freud._lib.autotune_report()


def test_rdf_frames_without_graphs(freud):
    frames = make_frames(freud, [900, 1800], 9)
    batch = freud.locality.FrameBatch(frames)
    freud._lib.set_graphs(False)
    try:
        a = freud.density.RDF(100, 2.0).compute(batch).bin_counts_u64
    finally:
        freud._lib.set_graphs(True)
    b = freud.density.RDF(100, 2.0).compute(batch).bin_counts_u64
    np.testing.assert_array_equal(a, b)


def test_rdf_frames_2d_and_unwrapped(freud):
    frames = make_frames(freud, [1500, 400, 2600], 3, is2d=True)
    ref = per_frame_rdf(freud, frames, 120, 3.0)
    rdf = freud.density.RDF(120, 3.0).compute(freud.locality.FrameBatch(frames))
    np.testing.assert_array_equal(rdf.bin_counts, ref.bin_counts)
    np.testing.assert_array_equal(rdf.rdf, ref.rdf)
    frames = make_frames(freud, [1500, 2600], 4, unwrapped=True)
    ref = per_frame_rdf(freud, frames, 120, 2.0)
    rdf = freud.density.RDF(120, 2.0).compute(freud.locality.FrameBatch(frames))
    np.testing.assert_array_equal(rdf.bin_counts, ref.bin_counts)


def test_rdf_frames_set_points(freud):
    frames = make_frames(freud, [1000, 2000], 21)
    moved = make_frames(freud, [1000, 2000], 22)
    batch = freud.locality.FrameBatch(frames)
    freud.density.RDF(80, 2.0).compute(batch)
    batch.set_points(np.concatenate([p for _, p in moved]))
    got = freud.density.RDF(80, 2.0).compute(batch).bin_counts
    # same boxes, new positions
    ref = per_frame_rdf(freud, [(frames[f][0], moved[f][1]) for f in range(2)], 80, 2.0)
    np.testing.assert_array_equal(got, ref.bin_counts)


def test_rdf_frames_from_device(freud):
    import torch

    frames = make_frames(freud, [1300, 600], 8)
    pts = np.concatenate([p for _, p in frames])
    t = torch.from_numpy(pts).cuda()
    offs = np.array([0, 1300, 1900], np.uint64)
    batch = freud.locality.FrameBatch.from_device([b for b, _ in frames], t.data_ptr(), offs, keepalive=t)
    got = freud.density.RDF(90, 2.2).compute(batch).bin_counts
    np.testing.assert_array_equal(got, per_frame_rdf(freud, frames, 90, 2.2).bin_counts)


def test_frames_errors(freud):
    box = freud.box.Box.cube(10.0)
    pts = np.zeros((5, 3), np.float32)
    with pytest.raises(ValueError):
        freud.locality.FrameBatch([(box, pts), (box, np.zeros((0, 3), np.float32))])
    with pytest.raises(ValueError):
        freud.locality.FrameBatch([])
    batch = freud.locality.FrameBatch([(box, pts)])
    with pytest.raises(RuntimeError):
        freud.density.RDF(10, 6.0).compute(batch)
    st = freud.order.Steinhardt(6)
    with pytest.raises(ValueError):
        st.compute(batch, neighbors={"num_neighbors": 4})
    with pytest.raises(ValueError):
        st.compute(batch)


@pytest.mark.parametrize("average,wl", [(True, False), (False, True)])
def test_steinhardt_frames_vs_fp64_oracle(freud, average, wl):
    """Ql within 1e-5 relative of the FP64 oracle per frame (Steinhardt l = 6 and
    l = 4, 6 with wl); Wl within 1e-5 (|w| + M) (M = sum of the magnitudes of
    the Wigner-3j terms); the per-frame system order within 1e-5 relative."""
    frames = make_frames(freud, [2000, 333, 1500, 90], 31)
    ls = [6] if not wl else [4, 6]
    st = freud.order.Steinhardt(ls if len(ls) > 1 else ls[0], average=average, wl=wl, wl_normalize=wl)
    st.compute(freud.locality.FrameBatch(frames), neighbors={"r_max": 1.5})
    ql = np.asarray(st.ql).reshape(-1, len(ls))
    po = np.asarray(st.particle_order).reshape(-1, len(ls))
    order = np.asarray(st.order).reshape(len(frames), len(ls))
    off = 0
    for f, (box, pts) in enumerate(frames):
        n = len(pts)
        ij, d, v = O.query(box, pts, r_max=1.5, exclude_ii=True, arith=O.ARITH_AABB)
        o = O.steinhardt(ls, box, pts, ij, d, average=average, wl=wl, wl_normalize=wl)
        qref = o["ql_ave"] if average else o["ql"]
        ok = np.isfinite(qref)
        np.testing.assert_allclose(ql[off:off + n][ok], qref[ok], rtol=1e-5, atol=1e-7)
        if wl:
            w, mag = o["wl"], o["wl_mag"]
            okw = np.isfinite(w)
            err = np.abs(po[off:off + n] - w)[okw]
            assert np.all(err <= 1e-5 * (np.abs(w[okw]) + mag[okw]))
        np.testing.assert_allclose(order[f], o["order"], rtol=1e-5)
        off += n


def test_steinhardt_frames_match_per_frame(freud):
    """Each frame of a batch against the same frame computed alone (different bond
    order within a particle, so float32 sums agree to rounding)."""
    frames = make_frames(freud, [2500, 700], 41)
    st = freud.order.Steinhardt(6, average=True)
    st.compute(freud.locality.FrameBatch(frames), neighbors={"r_max": 1.5})
    ql = np.asarray(st.ql)
    off = 0
    for f, (box, pts) in enumerate(frames):
        s1 = freud.order.Steinhardt(6, average=True).compute((box, pts), neighbors={"r_max": 1.5})
        np.testing.assert_allclose(ql[off:off + len(pts)], s1.ql, rtol=2e-6, atol=1e-7)
        np.testing.assert_allclose(np.asarray(st.order)[f], s1.order, rtol=2e-6)
        off += len(pts)


def test_rdf_states_of_frame_ranges_combine(freud):
    """Two RDFs over disjoint frame ranges (as two processes would hold them),
    combined on the host and loaded into a third: equal to one RDF over every frame."""
    from freud_gb300 import replicas

    frames = make_frames(freud, [900, 1400, 600, 1100, 750], 51)
    whole = per_frame_rdf(freud, frames, 70, 2.0)
    parts = []
    for r in range(2):
        lo, hi = replicas.frame_range(len(frames), r, 2)
        rdf = freud.density.RDF(70, 2.0)
        rdf.compute(freud.locality.FrameBatch(frames[lo:hi]), reset=False)
        parts.append(replicas.rdf_state(rdf))
    merged = replicas.load_rdf_state(freud.density.RDF(70, 2.0), replicas.combine_rdf_states(parts))
    np.testing.assert_array_equal(merged.bin_counts_u64, whole.bin_counts_u64)
    np.testing.assert_array_equal(merged.rdf, whole.rdf)
    np.testing.assert_array_equal(merged.n_r, whole.n_r)


def _clustered_frame(freud, seed, L=12.0, blobs=3, per_blob=300, sigma=0.35, background=500):
    """Dense Gaussian clusters (cells of well over 32 points, stencils of several
    hundred candidates) over a uniform background; 60 points moved up to 0.5
    outside the box (queries and candidates with a nonzero box image)."""
    rs = np.random.RandomState(seed)
    box = freud.box.Box.cube(L)
    centres = rs.uniform(-L / 2 + 1.5, L / 2 - 1.5, (blobs, 3))
    pts = np.concatenate([c + rs.normal(0, sigma, (per_blob, 3)) for c in centres]
                         + [rs.uniform(-L / 2, L / 2, (background, 3))])
    pts[-30:, 0] = rs.uniform(L / 2, L / 2 + 0.5, 30)
    pts[-60:-30, 1] = rs.uniform(-L / 2 - 0.5, -L / 2, 30)
    return box, pts.astype(np.float32)


@pytest.mark.parametrize("average", [False, True])
def test_steinhardt_ball_dense_cells_points_outside(freud, average):
    """Steinhardt l = 4, 6 on AABB ball neighbours (r_max 1.2) of clustered points,
    some outside the box, as one (box, points) call and inside a FrameBatch with a
    uniform frame: Ql within 1e-5 relative of the FP64 oracle per frame."""
    dense = _clustered_frame(freud, 71)
    uni = make_frames(freud, [1500], 72, tilt_every=1, unwrapped=True)[0]
    ls = [4, 6]
    one = freud.order.Steinhardt(ls, average=average).compute(dense, neighbors={"r_max": 1.2})
    st = freud.order.Steinhardt(ls, average=average)
    st.compute(freud.locality.FrameBatch([uni, dense]), neighbors={"r_max": 1.2})
    ql_b = np.asarray(st.ql).reshape(-1, 2)
    for ql, (box, pts) in ((np.asarray(one.ql).reshape(-1, 2), dense), (ql_b[:len(uni[1])], uni),
                           (ql_b[len(uni[1]):], dense)):
        ij, d, v = O.query(box, pts, r_max=1.2, exclude_ii=True, arith=O.ARITH_AABB)
        o = O.steinhardt(ls, box, pts, ij, d, average=average)
        qref = o["ql_ave"] if average else o["ql"]
        ok = np.isfinite(qref)
        assert np.array_equal(ok, np.isfinite(ql))
        np.testing.assert_allclose(ql[ok], qref[ok], rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("average", [False, True])
def test_steinhardt_frames_one_pass_after_two(freud, average):
    """Dense clusters: the bonds far exceed the uniform-density estimate, so the first
    batched call overflows the one-pass arrays and takes the two passes; the second
    call is sized by the first and runs in one pass, with cells of several candidate
    tiles counted then filled. Both give the same per-particle bonds in the same
    order, so the same Ql bit for bit, within 1e-5 of the FP64 oracle."""
    dense = _clustered_frame(freud, 81, blobs=4, per_blob=400)
    uni = make_frames(freud, [2000], 82)[0]
    st = freud.order.Steinhardt([4, 6], average=average)
    batch = freud.locality.FrameBatch([dense, uni])
    st.compute(batch, neighbors={"r_max": 1.2})
    first = np.asarray(st.ql).copy()
    st.compute(freud.locality.FrameBatch([dense, uni]), neighbors={"r_max": 1.2})
    second = np.asarray(st.ql)
    np.testing.assert_array_equal(first, second)
    box, pts = dense
    ij, d, v = O.query(box, pts, r_max=1.2, exclude_ii=True, arith=O.ARITH_AABB)
    o = O.steinhardt([4, 6], box, pts, ij, d, average=average)
    qref = o["ql_ave"] if average else o["ql"]
    ql = second.reshape(-1, 2)[:len(pts)]
    ok = np.isfinite(qref)
    assert np.array_equal(ok, np.isfinite(ql))
    np.testing.assert_allclose(ql[ok], qref[ok], rtol=1e-5, atol=1e-7)
