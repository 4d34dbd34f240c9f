"""GSD reader and the reference's trajectory known answers on the CPU: the reader
against byte-built files (both file-layer versions, frame-0 fallback, defaults,
malformed files) and, where the reference tree exists, against the fixture
generated from its files; the oracle against the Lennard-Jones RDF of
tests/integration/test_reader_integrations.py:34-41 and the GC Steinhardt values
of tests/validation/test_steinhardt_average.py:83-109."""

import os

import numpy as np
import pytest

from conftest import load_golden
from gsd_bytes import gsd_bytes, trajectory_bytes
from oracle import oracle as O

# the reference's test tree, when the environment names it (not on the GPU machine)
REF_TESTS = os.path.join(os.environ.get("FREUD_REFERENCE_DIR", ""), "tests") if os.environ.get(
    "FREUD_REFERENCE_DIR") else ""


def _gsd():
    from freud_gb300 import gsd

    return gsd


@pytest.mark.parametrize("version", [1, 2])
def test_reader_round_trip(tmp_path, version):
    gsd = _gsd()
    rs = np.random.RandomState(5)
    boxes = [(5.0, 6.0, 7.0, 0.1, 0.0, 0.2), (5.5, 6.0, 7.0, 0.0, 0.0, 0.0)]
    pos = [rs.random_sample((n, 3)).astype(np.float32) for n in (7, 9)]
    path = tmp_path / "t.gsd"
    path.write_bytes(trajectory_bytes(boxes, pos, dims=3, version=version))
    with gsd.open(str(path)) as traj:
        assert len(traj) == 2
        assert traj.gsd_version[0] == version
        assert "particles/position" in traj.names
        for f in range(2):
            fr = traj[f]
            np.testing.assert_array_equal(fr.particles.position, pos[f])
            np.testing.assert_array_equal(fr.configuration.box, np.float32(boxes[f]))
            assert fr.configuration.dimensions == 3  # stored in frame 0 only
            assert fr.configuration.step == 1000 * f
            assert fr.particles.N == len(pos[f])
        assert traj[-1].configuration.step == 1000
        assert [fr.particles.N for fr in traj] == [7, 9]
        with pytest.raises(IndexError):
            traj[2]


def test_reader_frame0_fallback_and_defaults(tmp_path):
    gsd = _gsd()
    p0 = np.arange(6, dtype=np.float32).reshape(2, 3)
    frames = [{"particles/N": np.array([2], np.uint32), "particles/position": p0},
              {"configuration/step": np.array([5], np.uint64)}]
    path = tmp_path / "d.gsd"
    path.write_bytes(gsd_bytes(frames))
    with gsd.open(str(path)) as traj:
        f1 = traj[1]
        np.testing.assert_array_equal(f1.particles.position, p0)  # taken from frame 0
        np.testing.assert_array_equal(f1.configuration.box, [1, 1, 1, 0, 0, 0])  # schema default
        assert f1.configuration.dimensions == 3 and f1.configuration.step == 5
        assert traj[0].configuration.step == 0


def test_reader_2d_frame_system(tmp_path):
    gsd = _gsd()
    pos = [np.array([[0.1, 0.2, 0.0], [1.0, -1.0, 0.0]], np.float32)]
    path = tmp_path / "p.gsd"
    path.write_bytes(trajectory_bytes([(4.0, 4.0, 1.0, 0.1, 0.3, 0.2)], pos, dims=2))
    with gsd.open(str(path)) as traj:
        box, pts = traj[0].system()
        np.testing.assert_array_equal(box, [4.0, 4.0, 0.0, np.float32(0.1), 0.0, 0.0])
        np.testing.assert_array_equal(pts, pos[0])
        from freud_gb300.locality import _as_box_points

        box2, pts2 = _as_box_points(traj[0])
        np.testing.assert_array_equal(box2, box)
        assert pts2 is traj[0].particles.position or np.array_equal(pts2, pts)


def test_reader_rejects_malformed(tmp_path):
    gsd = _gsd()
    good = trajectory_bytes([(3.0, 3.0, 3.0, 0, 0, 0)], [np.zeros((2, 3), np.float32)])
    cases = {
        "empty": b"",
        "short": good[:100],
        "magic": gsd_bytes([{"particles/N": np.array([0], np.uint32)}], magic=0x1234),
        "schema": gsd_bytes([{"particles/N": np.array([0], np.uint32)}], schema=b"other"),
        "truncated": good[:-8],
    }
    for name, data in cases.items():
        path = tmp_path / (name + ".gsd")
        path.write_bytes(data)
        with pytest.raises(RuntimeError):
            gsd.open(str(path))
    with pytest.raises(ValueError):
        gsd.open(str(tmp_path / "empty.gsd"), "wb")


@pytest.mark.skipif(not REF_TESTS or not os.path.isdir(REF_TESTS),
                    reason="FREUD_REFERENCE_DIR does not name the reference tree")
def test_reader_on_reference_files():
    gsd = _gsd()
    lj = load_golden("lj_traj")
    with gsd.open(os.path.join(REF_TESTS, "integration", "files", "lj", "lj.gsd")) as traj:
        assert len(traj) == len(lj["positions"])
        for f, fr in enumerate(traj):
            np.testing.assert_array_equal(fr.particles.position, lj["positions"][f])
            np.testing.assert_array_equal(fr.configuration.box, np.float32(lj["boxes"][f][:6]))
            assert fr.configuration.step == lj["steps"][f]
    gc = load_golden("gc_config")
    path = os.path.join(REF_TESTS, "validation", "files", "steinhardt_average", "Test_Configuration.gsd")
    with gsd.open(path) as traj:
        np.testing.assert_array_equal(traj[-1].particles.position, gc["positions"])


def test_oracle_lj_known_rdf():
    """RDF(bins=100, r_max=5) accumulated over the 10 Lennard-Jones frames: the
    oracle's counts equal the reference's bit for bit and its rdf the known
    answer within the reference test's tolerance (rtol = atol = 1e-5)."""
    lj = load_golden("lj_traj")
    counts = np.zeros(100, np.uint64)
    for b, p in zip(lj["boxes"], lj["positions"]):
        O.rdf_counts_query(tuple(b), p, 100, 5.0, counts=counts)
    np.testing.assert_array_equal(counts, lj["ref_counts"])
    b = lj["boxes"][-1]
    vol = np.float32(b[0]) * np.float32(b[1]) * np.float32(b[2])
    n = len(lj["positions"][-1])
    g, nr = O.rdf_reduce(counts, 5.0, 0.0, len(lj["boxes"]), n, n, vol)
    np.testing.assert_array_equal(g, lj["ref_rdf"])
    np.testing.assert_array_equal(nr, lj["ref_n_r"])
    np.testing.assert_allclose(g, lj["rdf_known"], rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("average", [False, True])
def test_oracle_gc_steinhardt(average):
    """q4, q6, w4, w6 (wl_normalize) on AABB ball neighbours r_max 1.4 of the GC
    configuration: the FP64 oracle within the reference test's atol 2e-5 of the GC
    code and within 2e-5 of the reference's float32 values."""
    gc = load_golden("gc_config")
    box = tuple(gc["box"])
    pts = gc["positions"]
    ij, d, _ = O.query(box, pts, r_max=1.4, exclude_ii=True)
    cols = []
    for l, wl in ((4, False), (6, False), (4, True), (6, True)):
        o = O.steinhardt([l], box, pts, ij, d, average=average, wl=wl, wl_normalize=wl)
        key = "wl" if wl else ("ql_ave" if average else "ql")
        cols.append(o[key][:, 0])
    got = np.stack(cols, 1)
    np.testing.assert_allclose(got, gc["gc_ave" if average else "gc"], atol=2e-5)
    np.testing.assert_allclose(got, gc["ref_ave" if average else "ref"], atol=2e-5)
