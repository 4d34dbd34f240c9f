"""The allocation-free RDF histogram entry point (fg_rdf_histogram_noalloc).

Callers that cannot allocate device memory (for example an analysis plugin that
runs inside a simulation engine which owns every device allocation) get the
same counts as the allocating RDF path. This file is collected last so that a
run stopping at the first failure has already run every other test; it passes
alone in a fresh process and after the other tests."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _counts_via_rdf(freud, L, lib, box, pts_dev, n, r_max, bins, kind):
    """The existing allocating path: fg_rdf_create + fg_rdf_accumulate_device."""
    nq = ctypes.c_void_p()
    lib.check(lib.lib.fg_nq_create_device(ctypes.byref(box), ctypes.c_void_p(pts_dev.data_ptr()), n, kind, 0.0,
                                          ctypes.byref(nq)))
    rdf = ctypes.c_void_p()
    lib.check(lib.lib.fg_rdf_create(bins, r_max, 0.0, ctypes.byref(rdf)))
    args = lib.make_args(lib.MODE_BALL, r_max=r_max, exclude_ii=True)
    lib.check(lib.lib.fg_rdf_accumulate_device(rdf, nq, None, n, None, ctypes.byref(args)))
    out = np.zeros(bins, np.uint64)
    lib.check(lib.lib.fg_rdf_get_u64(rdf, lib.ptr(out), None, None))
    lib.lib.fg_rdf_destroy(rdf)
    lib.lib.fg_nq_destroy(nq)
    return out


@pytest.mark.parametrize("kind", [0, 2])
def test_noalloc_matches_allocating_path_twice(kind):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import freud_gb300 as freud
    from freud_gb300 import _lib as lib

    bins, r_max = 120, 3.0
    out = torch.zeros(bins, dtype=torch.int64, device="cuda")
    for call, (L, n, seed) in enumerate([(24.0, 20000, 1), (18.0, 9000, 2)]):
        box, pts = freud.data.make_random_system(L, n, seed=seed)
        pts_dev = torch.from_numpy(np.ascontiguousarray(pts, np.float32)).cuda()
        cbox = box._c_box()
        lib.check(lib.lib.fg_rdf_histogram_noalloc(ctypes.byref(cbox), ctypes.c_void_p(pts_dev.data_ptr()), n,
                                                   r_max, 0.0, bins, 1, kind, ctypes.c_void_p(out.data_ptr()),
                                                   None))
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint64)
        want = _counts_via_rdf(freud, L, lib, cbox, pts_dev, n, r_max, bins, kind)
        np.testing.assert_array_equal(got, want, err_msg="call %d" % call)
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
