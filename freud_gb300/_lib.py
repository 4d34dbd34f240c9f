"""ctypes binding of libfreud_gb300.so (the C ABI declared in include/freud_gb300.h).

The library is built in-tree (freud_gb300/_build/). There is no CPU fallback:
if the library is missing this module raises ImportError, and calls that reach
the device raise RuntimeError when no GPU is available.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfreud_gb300.so")

FG_OK, FG_ERR_VALUE, FG_ERR_RUNTIME, FG_ERR_INDEX, FG_ERR_CUDA, FG_ERR_MEMORY = range(6)
MODE_NONE, MODE_BALL, MODE_NEAREST = 0, 1, 2
NQ_RAWPOINTS, NQ_AABB, NQ_LINKCELL, NQ_CELLQUERY = 0, 1, 2, 3
DEFAULT_NUM_NEIGHBORS = 0xFFFFFFFF


class fg_box(ctypes.Structure):
    _fields_ = [("Lx", ctypes.c_float), ("Ly", ctypes.c_float), ("Lz", ctypes.c_float),
                ("xy", ctypes.c_float), ("xz", ctypes.c_float), ("yz", ctypes.c_float),
                ("is2D", ctypes.c_int), ("periodic_x", ctypes.c_int), ("periodic_y", ctypes.c_int),
                ("periodic_z", ctypes.c_int)]


class fg_query_args(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("num_neighbors", ctypes.c_uint32), ("r_max", ctypes.c_float),
                ("r_min", ctypes.c_float), ("r_guess", ctypes.c_float), ("scale", ctypes.c_float),
                ("exclude_ii", ctypes.c_int)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "libfreud_gb300.so is not built (%s); run `python -m freud_gb300.build` "
            "(nvcc, sm_103a). There is no CPU fallback." % LIB_PATH)
    return ctypes.CDLL(LIB_PATH)


lib = _load()

P = ctypes.c_void_p
PP = ctypes.POINTER(ctypes.c_void_p)
u32, u64, f32, i32 = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float, ctypes.c_int
pu32, pu64, pf32 = ctypes.POINTER(u32), ctypes.POINTER(u64), ctypes.POINTER(f32)
pbox, pargs = ctypes.POINTER(fg_box), ctypes.POINTER(fg_query_args)

# name -> argtypes (restype is the int status unless listed in _RESTYPES)
SIGNATURES = {
    "fg_last_error": [],
    "fg_version": [],
    "fg_set_stream": [P],
    "fg_launch_count": [pu64],
    "fg_profile_enable": [i32],
    "fg_profile_report": [ctypes.c_char_p, ctypes.c_size_t],
    "fg_host_alloc": [ctypes.c_size_t, PP],
    "fg_host_free": [P],
    "fg_nq_create": [pbox, P, u32, i32, f32, PP],
    "fg_nq_create_device": [pbox, P, u32, i32, f32, PP],
    "fg_nq_destroy": [P],
    "fg_nq_cell_width": [P, pf32],
    "fg_nq_num_points": [P, pu32],
    "fg_nq_get_points": [P, P],
    "fg_nq_query": [P, P, u32, pargs, i32, PP],
    "fg_nq_query_device": [P, P, u32, pargs, i32, PP],
    "fg_nlist_from_arrays": [u64, P, u32, P, u32, P, P, PP],
    "fg_nlist_all_pairs": [pbox, P, u32, P, u32, i32, PP],
    "fg_nlist_destroy": [P],
    "fg_nlist_copy": [P, PP],
    "fg_nlist_num_bonds": [P, pu64],
    "fg_nlist_num_query_points": [P, pu32],
    "fg_nlist_num_points": [P, pu32],
    "fg_nlist_get": [P, P, P, P, P],
    "fg_nlist_device_arrays": [P, PP, PP, PP],
    "fg_nlist_segments": [P, P, P],
    "fg_nlist_find_first_index": [P, u32, pu32],
    "fg_nlist_filter": [P, P],
    "fg_nlist_filter_r": [P, f32, f32],
    "fg_nlist_sort": [P, i32],
    "fg_pmft_create": [i32, P, P, PP],
    "fg_pmft_destroy": [P],
    "fg_pmft_reset": [P],
    "fg_pmft_accumulate": [P, P, P, u32, P, u32, P, u32, P, u32, P, pargs],
    "fg_pmft_get": [P, P, P],
    "fg_pmft_axis": [P, i32, P, P, P, pu32],
    "fg_pmft_state": [P, pbox, pu32],
    "fg_cf_create": [u32, f32, PP],
    "fg_cf_destroy": [P],
    "fg_cf_reset": [P],
    "fg_cf_accumulate": [P, P, P, u32, P, u32, P, u32, P, pargs],
    "fg_cf_get": [P, P, P],
    "fg_cf_bin_edges": [P, P, P],
    "fg_cf_state": [P, pbox, pu32],
    "fg_rdf_create": [u32, f32, f32, PP],
    "fg_rdf_destroy": [P],
    "fg_rdf_set_mode": [P, i32],
    "fg_rdf_reset": [P],
    "fg_rdf_accumulate": [P, P, P, u32, P, pargs],
    "fg_rdf_accumulate_device": [P, P, P, u32, P, pargs],
    "fg_rdf_get": [P, P, P, P],
    "fg_rdf_get_u64": [P, P, P, P],
    "fg_rdf_bin_edges": [P, P, P],
    "fg_rdf_state": [P, pbox, pu32, pu32, pu32],
    "fg_rdf_set_state": [P, P, u32, pbox, u32, u32],
    "fg_steinhardt_create": [P, u32, i32, i32, i32, i32, PP],
    "fg_steinhardt_destroy": [P],
    "fg_steinhardt_compute": [P, P, P, pargs],
    "fg_steinhardt_num_particles": [P, pu32],
    "fg_steinhardt_get": [P, P, P, P, P],
    "fg_rdf_histogram_noalloc": [pbox, P, u32, f32, f32, u32, i32, i32, P, P],
    "fg_frames_create": [P, P, P, u32, PP],
    "fg_frames_create_device": [P, P, P, u32, PP],
    "fg_frames_set_points": [P, P],
    "fg_frames_create_list": [P, P, P, u32, PP],
    "fg_frames_destroy": [P],
    "fg_frames_info": [P, pu32, pu64],
    "fg_rdf_accumulate_frames": [P, P, pargs],
    "fg_steinhardt_compute_frames": [P, P, pargs],
    "fg_steinhardt_num_frames": [P, pu32],
    "fg_batch_set_config": [i32, i32, i32],
    "fg_autotune_report": [ctypes.c_char_p, ctypes.c_size_t],
    "fg_set_graphs": [i32],
    "fg_set_count_kernel": [i32],
    "fg_check_division": [u64, u64, pu64, P],
}
_RESTYPES = {"fg_last_error": ctypes.c_char_p, "fg_version": ctypes.c_int}

for _name, _args in SIGNATURES.items():
    _fn = getattr(lib, _name)
    _fn.argtypes = _args
    _fn.restype = _RESTYPES.get(_name, ctypes.c_int)


def check(status):
    """Raise the Python exception the reference's binding would raise."""
    if status == FG_OK:
        return
    msg = (lib.fg_last_error() or b"").decode(errors="replace")
    if status == FG_ERR_VALUE:
        raise ValueError(msg)
    if status == FG_ERR_INDEX:
        raise IndexError(msg)
    if status == FG_ERR_MEMORY:
        raise MemoryError(msg)
    raise RuntimeError(msg)


def ptr(a):
    """ctypes pointer to a numpy array's data (None passes through)."""
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def launch_count():
    out = u64()
    check(lib.fg_launch_count(ctypes.byref(out)))
    return int(out.value)


def profile_enable(on=True):
    check(lib.fg_profile_enable(int(bool(on))))


def profile_report():
    """{kernel name: (launches, total_ms)} since the last profile_enable()."""
    buf = ctypes.create_string_buffer(1 << 16)
    check(lib.fg_profile_report(buf, len(buf)))
    out = {}
    for line in buf.value.decode().splitlines():
        name, n, ms = line.rsplit(" ", 2)
        out[name] = (int(n), float(ms))
    return out


def autotune_report():
    buf = ctypes.create_string_buffer(1 << 16)
    check(lib.fg_autotune_report(buf, len(buf)))
    return buf.value.decode()


def set_batch_config(shell=0, warps=8, copies=1):
    """Force the batched RDF kernel's launch shape (shell=0: autotune)."""
    check(lib.fg_batch_set_config(int(shell), int(warps), int(copies)))


def set_graphs(enable):
    check(lib.fg_set_graphs(int(bool(enable))))


def set_count_kernel(which):
    """0: automatic choice of the NeighborList count pass; 1: block per cell with
    lanes over candidates everywhere (both give the same lists)."""
    check(lib.fg_set_count_kernel(int(which)))


def set_stream(stream_ptr):
    check(lib.fg_set_stream(ctypes.c_void_p(stream_ptr) if stream_ptr else None))


def make_args(mode=MODE_NONE, num_neighbors=DEFAULT_NUM_NEIGHBORS, r_max=-1.0, r_min=0.0, r_guess=-1.0,
              scale=-1.0, exclude_ii=False):
    a = fg_query_args()
    a.mode = int(mode)
    a.num_neighbors = int(num_neighbors) & 0xFFFFFFFF
    a.r_max = float(r_max)
    a.r_min = float(r_min)
    a.r_guess = float(r_guess)
    a.scale = float(scale)
    a.exclude_ii = int(bool(exclude_ii))
    return a


class Handle:
    """Owns one opaque library handle and destroys it with the given function."""

    __slots__ = ("value", "_destroy")

    def __init__(self, value, destroy):
        self.value = value
        self._destroy = destroy

    def __del__(self):
        v, self.value = self.value, None
        if v is not None and lib is not None:
            try:
                self._destroy(v)
            except Exception:  # interpreter shutdown
                pass


# ---- page-locked host arrays -----------------------------------------------------
# Blocks of page-locked memory, pooled by size: a NeighborList read back to the host
# lands in one (DMA at the link's rate), and returns to the pool when the last array
# viewing it is dropped. The pool keeps at most _PINNED_KEEP bytes.

_PINNED_KEEP = 16 << 30
_pinned_free = {}
_pinned_pooled = 0


class _PinnedBlock:
    __slots__ = ("addr", "nbytes")

    def __init__(self, addr, nbytes):
        self.addr = addr
        self.nbytes = nbytes

    def __del__(self):
        global _pinned_pooled
        try:
            if _pinned_pooled + self.nbytes <= _PINNED_KEEP:
                _pinned_free.setdefault(self.nbytes, []).append(self.addr)
                _pinned_pooled += self.nbytes
            else:
                lib.fg_host_free(ctypes.c_void_p(self.addr))
        except Exception:  # interpreter shutdown
            pass


def pinned_empty(shape, dtype):
    """An uninitialised numpy array in page-locked host memory (pooled)."""
    import numpy as np

    global _pinned_pooled
    dtype = np.dtype(dtype)
    count = 1
    for s in (shape if isinstance(shape, tuple) else (shape,)):
        count *= int(s)
    need = max(count * dtype.itemsize, 1)
    nbytes = (need + (2 << 20) - 1) // (2 << 20) * (2 << 20)
    free = _pinned_free.get(nbytes)
    if free:
        addr = free.pop()
        _pinned_pooled -= nbytes
    else:
        out = ctypes.c_void_p()
        check(lib.fg_host_alloc(nbytes, ctypes.byref(out)))
        addr = out.value
    raw = (ctypes.c_char * need).from_address(addr)
    raw._owner = _PinnedBlock(addr, nbytes)
    return np.frombuffer(raw, dtype=dtype, count=count).reshape(shape)
