"""Steinhardt order parameters, API-compatible with freud.order.Steinhardt
(freud/order.py:375-643). Ylm, qlm, averaging and Wl run on the GPU."""

import collections.abc
import ctypes

import numpy as np

from . import _lib
from .locality import FrameBatch, NeighborList, _QueryArgs, _PairCompute
from .util import _Compute


class Steinhardt(_PairCompute):
    """Rotationally invariant Steinhardt q_l / w_l for each particle.

    Args:
        l (unsigned int or sequence of unsigned int): spherical-harmonic degrees.
        average (bool): average qlm over the first neighbour shell (Lechner-Dellago).
        wl (bool): compute the third-order invariant w_l.
        weighted (bool): weight neighbours by the NeighborList weights.
        wl_normalize (bool): normalise w_l.
    """

    def __init__(self, l, average=False, wl=False, weighted=False, wl_normalize=False):
        if not isinstance(l, collections.abc.Sequence):
            l = [l]
        if len(l) == 0:
            raise ValueError("At least one l must be specified.")
        self._ls = [int(x) for x in l]
        ls = np.asarray(self._ls, dtype=np.uint32)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib.fg_steinhardt_create(_lib.ptr(ls), len(ls), int(average), int(wl), int(weighted),
                                                 int(wl_normalize), ctypes.byref(h)))
        self._handle = _lib.Handle(h, _lib.lib.fg_steinhardt_destroy)
        self._average, self._wl, self._weighted, self._wl_normalize = (bool(average), bool(wl), bool(weighted),
                                                                       bool(wl_normalize))
        self._cache = None

    @property
    def _h(self):
        return self._handle.value

    @property
    def average(self):
        return self._average

    @property
    def wl(self):
        return self._wl

    @property
    def weighted(self):
        return self._weighted

    @property
    def wl_normalize(self):
        return self._wl_normalize

    @property
    def l(self):
        return self._ls[0] if len(self._ls) == 1 else list(self._ls)

    def compute(self, system, neighbors=None):
        if isinstance(system, FrameBatch):
            # every frame with its own ball query; order is per frame
            if neighbors is None or isinstance(neighbors, NeighborList):
                raise ValueError("a FrameBatch needs ball query arguments as neighbors, e.g. {'r_max': 1.5}")
            query_args = dict(neighbors)
            query_args.setdefault("exclude_ii", True)
            qargs = _QueryArgs.from_dict(query_args)
            _lib.check(_lib.lib.fg_steinhardt_compute_frames(self._h, system._h, ctypes.byref(qargs._c())))
            self._cache = None
            return self
        nq, nlist, qargs, _qp, _nqp = self._preprocess_arguments(system, neighbors=neighbors)
        _lib.check(_lib.lib.fg_steinhardt_compute(self._h, nq._h, None if nlist is None else nlist._h,
                                                  ctypes.byref(qargs._c())))
        self._cache = None
        return self

    def _dims(self):
        n = ctypes.c_uint32()
        _lib.check(_lib.lib.fg_steinhardt_num_particles(self._h, ctypes.byref(n)))
        nf = ctypes.c_uint32()
        _lib.check(_lib.lib.fg_steinhardt_num_frames(self._h, ctypes.byref(nf)))
        return n.value, nf.value, len(self._ls)

    # outputs of at least this many bytes are read into page-locked arrays from the
    # library's pool (the device-to-host copy then runs by DMA)
    _PINNED_BYTES = 1 << 20

    def _fetch(self, key):
        """One output array, copied from the device on first access after a compute
        (every element is written by the copy)."""
        if self._cache is None:
            self._cache = {}
        if key in self._cache:
            return self._cache[key]
        n, nf, nl = self._dims()

        def empty(shape):
            count = int(np.prod(shape))
            return (_lib.pinned_empty if 4 * count >= self._PINNED_BYTES else np.empty)(shape, np.float32)

        if key == "ql":
            out = empty((n, nl))
            _lib.check(_lib.lib.fg_steinhardt_get(self._h, _lib.ptr(out), None, None, None))
        elif key == "po":
            out = empty((n, nl))
            _lib.check(_lib.lib.fg_steinhardt_get(self._h, None, _lib.ptr(out), None, None))
        elif key == "order":
            out = np.zeros(nf * nl, np.float32)
            _lib.check(_lib.lib.fg_steinhardt_get(self._h, None, None, None, _lib.ptr(out)))
            if nf > 1:
                out = out.reshape(nf, nl)
        else:
            stride = sum(2 * l + 1 for l in self._ls)
            qlm = empty((n * stride * 2,))
            _lib.check(_lib.lib.fg_steinhardt_get(self._h, None, None, _lib.ptr(qlm), None))
            qc = qlm.view(np.complex64)
            out, off = [], 0
            for l in self._ls:
                m = 2 * l + 1
                out.append(qc[off:off + n * m].reshape(n, m))
                off += n * m
        self._cache[key] = out
        return out

    @_Compute._computed_property
    def order(self):
        order = self._fetch("order")
        if order.ndim == 2:
            return order[:, 0] if order.shape[1] == 1 else order
        return order[0] if len(order) == 1 else order

    @_Compute._computed_property
    def particle_order(self):
        p = self._fetch("po")
        return np.ravel(p) if p.shape[1] == 1 else p

    @_Compute._computed_property
    def ql(self):
        q = self._fetch("ql")
        return np.ravel(q) if q.shape[1] == 1 else q

    @_Compute._computed_property
    def particle_harmonics(self):
        qlm = self._fetch("qlm")
        return qlm if len(qlm) > 1 else qlm[0]

    def __repr__(self):
        return ("freud.order.{}(l={}, average={}, wl={}, weighted={}, wl_normalize={})".format(
            type(self).__name__, self.l, self.average, self.wl, self.weighted, self.wl_normalize))
