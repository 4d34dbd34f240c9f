"""Several GPUs, one process each.

The path has no exchange step: frames are independent and an RDF over frames only
sums bin counts. So work is split as contiguous frame ranges, one per process, and
the accumulated RDF states are combined on the host afterwards - a few KB, no
device collective. freud's BondHistogramCompute keeps the last frame's box and N
next to the counts (BondHistogramCompute.h:115-126); the combination keeps those
of the last non-empty range, so the result equals one process accumulating every
frame in order.
"""

from collections import namedtuple
import ctypes

import numpy as np

RDFState = namedtuple("RDFState", ["counts", "n_frames", "box", "n_points", "n_query"])


def frame_range(n_frames, rank, world):
    """Contiguous frame range [lo, hi) of one rank; ranges cover every frame once
    and differ in length by at most one."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(int(n_frames), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def combine_rdf_states(states):
    """States in rank (frame) order -> one state: counts and frame counters summed,
    box and N of the last state that holds frames."""
    states = list(states)
    if not states:
        raise ValueError("no states to combine")
    counts = np.zeros_like(np.asarray(states[0].counts, dtype=np.uint64))
    frames = 0
    last = None
    for st in states:
        counts += np.asarray(st.counts, dtype=np.uint64)
        frames += int(st.n_frames)
        if st.n_frames > 0:
            last = st
    last = last or states[-1]
    return RDFState(counts, frames, tuple(last.box), int(last.n_points), int(last.n_query))


def allgather_rdf_state(state, group=None):
    """Combination of every rank's state (torch.distributed, any backend)."""
    import torch.distributed as dist

    gathered = [None] * dist.get_world_size(group)
    dist.all_gather_object(gathered, tuple(state), group=group)
    return combine_rdf_states(RDFState(*g) for g in gathered)


def rdf_state(rdf):
    """The accumulated state of an RDF object (device counts read back)."""
    from . import _lib

    b = _lib.fg_box()
    nf, npts, nq = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
    _lib.check(_lib.lib.fg_rdf_state(rdf._h, ctypes.byref(b), ctypes.byref(nf), ctypes.byref(npts), ctypes.byref(nq)))
    counts = np.zeros(rdf.nbins, np.uint64)
    _lib.check(_lib.lib.fg_rdf_get_u64(rdf._h, _lib.ptr(counts), None, None))
    box = (b.Lx, b.Ly, b.Lz, b.xy, b.xz, b.yz, int(b.is2D))
    return RDFState(counts, nf.value, box, npts.value, nq.value)


def load_rdf_state(rdf, state):
    """Make rdf hold a (combined) state: its rdf, n_r and bin counts then come out
    as if it had accumulated every frame itself."""
    from . import _lib

    counts = np.ascontiguousarray(state.counts, dtype=np.uint64)
    if len(counts) != rdf.nbins:
        raise ValueError("bin count mismatch")
    Lx, Ly, Lz, xy, xz, yz, is2d = state.box
    b = _lib.fg_box(Lx, Ly, Lz, xy, xz, yz, int(is2d), 1, 1, 1)
    _lib.check(_lib.lib.fg_rdf_set_state(rdf._h, _lib.ptr(counts), int(state.n_frames), ctypes.byref(b),
                                         int(state.n_points), int(state.n_query)))
    rdf._has_computed = True
    return rdf
