"""Minimal stand-in for numba, used only by the oracle to import the reference.

This is test infrastructure. It lets the pure-Python reference implementation of
fteikpy be imported in an environment without numba, in the same mode the
reference's own CI runs its tests (``NUMBA_DISABLE_JIT=1``,
``.github/workflows/ci.yml:29``): ``jit`` returns the function unchanged and
``prange`` is ``range``. Nothing in the product imports this module.
"""

_num_threads = 1


def jit(*args, **kwargs):
    """Identity decorator that accepts both ``@jit`` and ``@jit(signature, ...)``."""
    if args and callable(args[0]):
        return args[0]

    def wrap(fn):
        return fn

    return wrap


njit = jit
prange = range


def get_num_threads():
    return _num_threads


def set_num_threads(n):
    global _num_threads
    _num_threads = int(n)
