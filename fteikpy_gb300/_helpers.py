"""Thread-count knobs kept for API compatibility (fteikpy/_helpers.py:4-27).

The reference sizes numba's CPU thread pool with them. Here the work runs on
the GPU, so the value is only stored and returned.
"""

_num_threads = 1


def get_num_threads():
    """Get current number of threads."""
    return _num_threads


def set_num_threads(n):
    """Set number of threads."""
    global _num_threads
    _num_threads = int(n)
