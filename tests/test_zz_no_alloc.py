"""The allocation-free RDF histogram entry point (fg_rdf_histogram_noalloc).

Callers that cannot allocate device memory (for example an analysis plugin that
runs inside a simulation engine which owns every device allocation) get the
same counts as the allocating RDF path and as the oracle. Each case makes two
calls in a row on different systems (the shared scratch keeps the previous
call's contents). This file is collected last so that a run stopping at the
first failure has already run every other test; it passes alone in a fresh
process and after the other tests."""

import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _counts_via_rdf(lib, box, pts_dev, n, r_max, r_min, bins, kind):
    """The existing allocating path: fg_rdf_create + fg_rdf_accumulate_device."""
    nq = ctypes.c_void_p()
    lib.check(lib.lib.fg_nq_create_device(ctypes.byref(box), ctypes.c_void_p(pts_dev.data_ptr()), n, kind, 0.0,
                                          ctypes.byref(nq)))
    rdf = ctypes.c_void_p()
    lib.check(lib.lib.fg_rdf_create(bins, r_max, r_min, ctypes.byref(rdf)))
    args = lib.make_args(lib.MODE_BALL, r_max=r_max, exclude_ii=True)
    lib.check(lib.lib.fg_rdf_accumulate_device(rdf, nq, None, n, None, ctypes.byref(args)))
    out = np.zeros(bins, np.uint64)
    lib.check(lib.lib.fg_rdf_get_u64(rdf, lib.ptr(out), None, None))
    lib.lib.fg_rdf_destroy(rdf)
    lib.lib.fg_nq_destroy(nq)
    return out


def _system(freud, shape, seed):
    """uniform: 20,000 points in a cube of side 24; triclinic: 15,000 in a tilted
    box; cluster: 12,000 uniform points plus a tight 3,000-point cluster, whose
    stencils exceed one candidate tile."""
    rs = np.random.RandomState(seed)
    if shape == "uniform":
        box = freud.box.Box.cube(24.0)
        f = rs.random_sample((20000, 3))
    elif shape == "triclinic":
        box = freud.box.Box(21.0, 22.0, 23.0, 0.3, -0.2, 0.1)
        f = rs.random_sample((15000, 3))
    else:
        box = freud.box.Box.cube(24.0)
        f = rs.random_sample((12000, 3))
    pts = box.make_absolute(f).astype(np.float32)
    if shape == "cluster":
        c = (rs.normal(0.0, 0.6, (3000, 3)) + np.array([2.0, -3.0, 1.0])).astype(np.float32)
        pts = np.concatenate([pts, c]).astype(np.float32)
    return box, pts


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("r_min", [0.0, 0.5])
@pytest.mark.parametrize("bins", [120, 5000])
def test_noalloc_matches_allocating_path_and_oracle(kind, r_min, bins):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import freud_gb300 as freud
    from freud_gb300 import _lib as lib

    r_max = 3.0
    arith = O.ARITH_WRAP if kind == 2 else O.ARITH_AABB
    out = torch.zeros(bins, dtype=torch.int64, device="cuda")
    for call, (shape, seed) in enumerate([("triclinic", 1), ("cluster", 2), ("uniform", 3)][:2 + (bins == 120)]):
        box, pts = _system(freud, shape, seed)
        n = len(pts)
        pts_dev = torch.from_numpy(np.ascontiguousarray(pts, np.float32)).cuda()
        cbox = box._c_box()
        lib.check(lib.lib.fg_rdf_histogram_noalloc(ctypes.byref(cbox), ctypes.c_void_p(pts_dev.data_ptr()), n,
                                                   r_max, r_min, bins, 1, kind, ctypes.c_void_p(out.data_ptr()),
                                                   None))
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint64).copy()
        want = _counts_via_rdf(lib, cbox, pts_dev, n, r_max, r_min, bins, kind)
        np.testing.assert_array_equal(got, want, err_msg="call %d (%s)" % (call, shape))
        oracle = O.rdf_counts_query(box, pts, bins, r_max, r_min=r_min, arith=arith)
        np.testing.assert_array_equal(got, oracle, err_msg="call %d (%s) vs oracle" % (call, shape))
        assert got.sum() > 0


def test_noalloc_rejects_too_many_points():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import freud_gb300 as freud
    from freud_gb300 import _lib as lib

    box = freud.box.Box.cube(100.0)
    n = (1 << 16) + 1
    pts = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    out = torch.zeros(10, dtype=torch.int64, device="cuda")
    st = lib.lib.fg_rdf_histogram_noalloc(ctypes.byref(box._c_box()), ctypes.c_void_p(pts.data_ptr()), n, 3.0, 0.0,
                                          10, 1, 2, ctypes.c_void_p(out.data_ptr()), None)
    assert st == lib.FG_ERR_VALUE
    assert b"65536" in lib.lib.fg_last_error()
