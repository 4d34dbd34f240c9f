"""Thread-count control, API-compatible with freud.parallel (freud/parallel.py:24-59).

The computation runs on the GPU, so the host thread count only affects host-side
helpers; the settings are recorded for API compatibility.
"""

import os

_num_threads = 0


def get_num_threads():
    """Number of host threads freud would use (0 means all cores)."""
    return _num_threads or (os.cpu_count() or 1)


def set_num_threads(nthreads=None):
    global _num_threads
    if nthreads is None or nthreads == 0:
        _num_threads = 0
    elif nthreads < 0:
        raise ValueError("nthreads must be a positive number")
    else:
        _num_threads = int(nthreads)


class NumThreads:
    """Context manager that sets the thread count within its block."""

    def __init__(self, N=None):
        self.restore_N = _num_threads
        self.N = N

    def __enter__(self):
        set_num_threads(self.N)
        return self

    def __exit__(self, *args):
        set_num_threads(self.restore_N)
