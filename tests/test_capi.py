"""CPU tests of the C-ABI boundary: the library builds for sm_103a, loads, exports
every entry point include/*.h declares, and reports device errors as exceptions
(no CPU fallback). No compute calls are made here."""

import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(fg_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("fg_nq_create", "fg_nq_query", "fg_rdf_accumulate", "fg_steinhardt_compute", "fg_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from freud_gb300 import _lib

    for name in declared_symbols():
        assert hasattr(_lib.lib, name), name
        assert name in _lib.SIGNATURES, name


def test_library_is_built_for_sm103a():
    from freud_gb300 import build

    assert "arch=compute_103a,code=sm_103a" in " ".join(build.NVCC_FLAGS)
    assert os.path.exists(build.LIB)


def test_validation_errors_without_device():
    """Argument validation that needs no device runs on the host and maps to the
    reference's exception classes."""
    from freud_gb300 import _lib

    out = ctypes.c_void_p()
    assert _lib.lib.fg_rdf_create(0, 1.0, 0.0, ctypes.byref(out)) == _lib.FG_ERR_VALUE
    assert b"nonzero number of bins" in _lib.lib.fg_last_error()
    assert _lib.lib.fg_rdf_create(10, -1.0, 0.0, ctypes.byref(out)) == _lib.FG_ERR_VALUE
    assert _lib.lib.fg_rdf_create(10, 1.0, 2.0, ctypes.byref(out)) == _lib.FG_ERR_VALUE
    box = _lib.fg_box(10, 10, 10, 0, 0, 0, 0, 1, 1, 1)
    assert _lib.lib.fg_nq_create(ctypes.byref(box), None, 0, 0, 0.0, ctypes.byref(out)) == _lib.FG_ERR_VALUE
    assert b"0 particles" in _lib.lib.fg_last_error()
    with pytest.raises(ValueError):
        _lib.check(_lib.FG_ERR_VALUE)


def test_device_calls_fail_loudly_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np

    import freud_gb300 as freud

    box, pts = freud.data.make_random_system(10, 50, seed=0)
    with pytest.raises(RuntimeError):
        freud.AABBQuery(box, pts)
