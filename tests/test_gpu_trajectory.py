"""The reference's trajectory known answers on the GPU, through the GSD reader
(the fixtures are rewritten as GSD files and read back, as the reference's
tests read theirs):

* tests/integration/test_reader_integrations.py:34-41 - RDF(bins=100, r_max=5)
  accumulated over the 10 Lennard-Jones frames with Steinhardt(6) on 6 nearest
  neighbours per frame; rdf within rtol = atol = 1e-5 of the known answer, and
  counts / rdf / n_r bit-identical to the reference's CPU code;
* tests/validation/test_steinhardt_average.py:83-109 - q4, q6, w4, w6 on AABB
  ball neighbours (r_max 1.4, exclude_ii) of the GC configuration, plain and
  averaged, within the reference test's atol 2e-5 of the GC code."""

import numpy as np
import pytest

from conftest import load_golden
from gsd_bytes import trajectory_bytes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _lj_file(tmp_path):
    lj = load_golden("lj_traj")
    path = tmp_path / "lj.gsd"
    path.write_bytes(trajectory_bytes(lj["boxes"], lj["positions"], dims=3, version=1))
    return lj, str(path)


def test_lj_run_analyses(freud, tmp_path):
    lj, path = _lj_file(tmp_path)
    rdf = freud.density.RDF(bins=100, r_max=5)
    ql = freud.order.Steinhardt(6)
    with freud.gsd.open(path) as traj:
        for system in traj:
            rdf.compute(system, reset=False)
            ql.compute(system, neighbors={"num_neighbors": 6})
    np.testing.assert_allclose(rdf.rdf, lj["rdf_known"], rtol=1e-5, atol=1e-5)
    np.testing.assert_array_equal(rdf.bin_counts, lj["ref_counts"])
    np.testing.assert_array_equal(rdf.rdf, lj["ref_rdf"])
    np.testing.assert_array_equal(rdf.n_r, lj["ref_n_r"])
    # Steinhardt of the last frame: reference float32 and FP64 oracle
    q6 = np.asarray(ql.particle_order).reshape(-1)
    np.testing.assert_allclose(q6, lj["ref_q6_last"], rtol=1e-5, atol=1e-6)
    b, p = tuple(lj["boxes"][-1]), lj["positions"][-1]
    ij, d, _ = O.query(b, p, num_neighbors=6, exclude_ii=True)
    o = O.steinhardt([6], b, p, ij, d)
    np.testing.assert_allclose(q6, o["ql"][:, 0], rtol=1e-5)


def test_lj_frame_batch(freud, tmp_path):
    """The whole trajectory as one FrameBatch: the same counts, rdf and n_r."""
    lj, path = _lj_file(tmp_path)
    with freud.gsd.open(path) as traj:
        batch = freud.locality.FrameBatch(traj)
    assert batch.num_frames == len(lj["boxes"])
    rdf = freud.density.RDF(bins=100, r_max=5).compute(batch, reset=False)
    np.testing.assert_array_equal(rdf.bin_counts, lj["ref_counts"])
    np.testing.assert_array_equal(rdf.rdf, lj["ref_rdf"])
    np.testing.assert_array_equal(rdf.n_r, lj["ref_n_r"])


@pytest.mark.parametrize("average", [False, True])
def test_gc_steinhardt(freud, tmp_path, average):
    gc = load_golden("gc_config")
    b = gc["box"]
    path = tmp_path / "gc.gsd"
    path.write_bytes(trajectory_bytes([b[:6]], [gc["positions"]], dims=3, version=2))
    with freud.gsd.open(str(path)) as traj:
        frame = traj[-1]
    nq = freud.locality.AABBQuery.from_system(frame)
    nlist = nq.query(frame.particles.position, dict(mode="ball", r_max=1.4, exclude_ii=True)).toNeighborList()
    cols = []
    for kw in (dict(l=4), dict(l=6), dict(l=4, wl=True, wl_normalize=True), dict(l=6, wl=True, wl_normalize=True)):
        op = freud.order.Steinhardt(average=average, weighted=False, **kw)
        op.compute(frame, neighbors=nlist)
        cols.append(np.asarray(op.particle_order).reshape(-1))
    got = np.stack(cols, 1)
    np.testing.assert_allclose(got, gc["gc_ave" if average else "gc"], atol=2e-5)
    np.testing.assert_allclose(got, gc["ref_ave" if average else "ref"], atol=2e-5)
