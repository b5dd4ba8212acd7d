"""ctypes front-end of the CPU oracle (``oracle/fteik_oracle.c``).

TEST INFRASTRUCTURE ONLY: used by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU legs of ``bench.py`` as the checker and the timed CPU baseline. The
product package never imports this module.

The functions mirror the reference's numba entry points
(``fteikpy/_fteik/_fteik3d.py:516-525`` ``solve3d``,
``fteikpy/_fteik/_fteik2d.py:667-674`` ``solve2d``, ``fteikpy/_interp/*``,
``fteikpy/_fteik/_ray*.py``) and take/return NumPy arrays.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfteik_oracle.so")
# The same source compiled for timing only, with the floating-point licences
# of the reference's numba build (fteikpy/_common.py:12: contract, arcp, nsz,
# afn): the CPU baseline of the benchmark, never a parity checker.
FAST_LIB_PATH = os.path.join(HERE, "_build", "libfteik_oracle_fast.so")

_libs = {}

_D = ctypes.c_double
_I = ctypes.c_int
_L = ctypes.c_long
_P = ctypes.c_void_p


def build():
    """Compile the oracle shared library (gcc, IEEE semantics, OpenMP)."""
    subprocess.check_call(["sh", os.path.join(HERE, "build_oracle.sh")])


def lib(fast=False):
    """The bitwise oracle library, or with ``fast`` the timing build."""
    path = FAST_LIB_PATH if fast else LIB_PATH
    L = _libs.get(path)
    if L is None:
        src_time = max(os.path.getmtime(os.path.join(HERE, f))
                       for f in ("fteik_oracle.c", "build_oracle.sh"))
        if not os.path.exists(path) or os.path.getmtime(path) < src_time:
            build()
        L = ctypes.CDLL(path)
        L.oracle_fteik3d_many.argtypes = [_P, _I, _I, _I, _D, _D, _D, _P, _I, _I, _I, _P, _P, _P, _I]
        L.oracle_fteik3d_many.restype = _I
        L.oracle_fteik3d_record.argtypes = [_P, _I, _I, _I, _D, _D, _D, _D, _D, _D, _I, _P, _P, _P, _P]
        L.oracle_fteik3d_record.restype = _I
        L.oracle_fteik3d_probe.argtypes = [_P, _I, _I, _I, _D, _D, _D, _P, _I, _I, _D, _P, _P,
                                           _P, _P, _I]
        L.oracle_fteik3d_probe.restype = _I
        L.oracle_adjoint3d.argtypes = [_P, _I, _I, _I, _D, _D, _D, _P, _I, _I, _P, _I, _P, _P, _I]
        L.oracle_adjoint3d.restype = _I
        L.oracle_fteik2d_many.argtypes = [_P, _I, _I, _D, _D, _P, _I, _I, _I, _P, _P, _P, _I]
        L.oracle_fteik2d_many.restype = _I
        L.oracle_interp3d.argtypes = [_P, _I, _P, _I, _P, _I, _P, _L, _P, _I, _D, _P]
        L.oracle_interp2d.argtypes = [_P, _I, _P, _I, _P, _L, _P, _I, _D, _P]
        L.oracle_vinterp3d.argtypes = [_P, _I, _P, _I, _P, _I, _P, _P, _I, _P, _D, _D, _P]
        L.oracle_vinterp2d.argtypes = [_P, _I, _P, _I, _P, _P, _I, _P, _D, _D, _P]
        L.oracle_ray3d.argtypes = [_P, _I, _P, _I, _P, _I, _P, _P, _I, _P, _D, _I, _I, _P, _P, _P]
        L.oracle_ray2d.argtypes = [_P, _I, _P, _I, _P, _P, _I, _P, _D, _I, _I, _P, _P, _P]
        _libs[path] = L
    return L


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def solve3d(slow, gridsize, sources, nsweep=2, grad=False, nthreads=None, fast=False):
    """Batched 3D solve. ``sources`` is (nsrc, 3), relative to the grid origin.
    ``fast`` runs the timing build (not bitwise).

    Returns (tt[nsrc, nz+1, nx+1, ny+1], ttgrad[nsrc, ..., 3] or None, vzero[nsrc]).
    """
    slow = _c(slow)
    src = _c(np.atleast_2d(sources))
    nz, nx, ny = slow.shape
    nsrc = len(src)
    tt = np.empty((nsrc, nz + 1, nx + 1, ny + 1))
    tg = np.empty((nsrc, nz + 1, nx + 1, ny + 1, 3)) if grad else np.empty(1)
    vz = np.empty(nsrc)
    nthreads = nthreads or os.cpu_count()
    st = lib(fast).oracle_fteik3d_many(
        _p(slow), nz, nx, ny, *map(float, gridsize), _p(src), nsrc, int(nsweep), int(grad),
        _p(tt), _p(tg), _p(vz), int(nthreads),
    )
    if st == 1:
        raise ValueError("source out of bound")
    return tt, (tg if grad else None), vz


def solve3d_record(slow, gridsize, source, nsweep=2):
    """One 3D solve with gradients that also returns the branch record (the
    reference's ttsgn) as int8 [nz+1, nx+1, ny+1, 3]."""
    slow = _c(slow)
    nz, nx, ny = slow.shape
    tt = np.empty((nz + 1, nx + 1, ny + 1))
    tg = np.empty((nz + 1, nx + 1, ny + 1, 3))
    sgn = np.zeros((nz + 1, nx + 1, ny + 1, 3), dtype=np.int8)
    vz = np.empty(1)
    st = lib().oracle_fteik3d_record(
        _p(slow), nz, nx, ny, *map(float, gridsize), *map(float, source), int(nsweep), _p(tt),
        _p(tg), _p(vz), _p(sgn),
    )
    if st == 1:
        raise ValueError("source out of bound")
    return tt, tg, float(vz[0]), sgn


def solve3d_probe(slow, gridsize, sources, nsweep=2, margin=0.0, tied=True, nthreads=None):
    """``solve3d`` (no gradients) that also returns, per source, a digest of
    every discrete decision of the sweeps (the candidate each node update
    keeps and the slowness cells attaining its operator's minimum), and the
    cells that a kept operator's minimum takes within a relative ``margin``
    of another cell (ties: one-sided derivatives there).

    Returns (tt, vzero, digests[nsrc] uint64, tied[nz, nx, ny] bool or None).
    Test infrastructure for choosing finite-difference cells of the adjoint
    check; it is not a restatement of a reference function."""
    slow = _c(slow)
    src = _c(np.atleast_2d(sources))
    nz, nx, ny = slow.shape
    nsrc = len(src)
    tt = np.empty((nsrc, nz + 1, nx + 1, ny + 1))
    vz = np.empty(nsrc)
    dig = np.zeros(nsrc, dtype=np.uint64)
    t = np.zeros(slow.shape, dtype=np.uint8) if tied else None
    st = lib().oracle_fteik3d_probe(
        _p(slow), nz, nx, ny, *map(float, gridsize), _p(src), nsrc, int(nsweep), float(margin),
        _p(tt), _p(vz), _p(dig), _p(t) if tied else None, int(nthreads or os.cpu_count()),
    )
    if st == 1:
        raise ValueError("source out of bound")
    return tt, vz, dig, (t.astype(bool) if tied else None)


def adjoint3d(slow, gridsize, sources, nsweep, receivers, grad_tt_rec, nthreads=None):
    """d(loss)/d(slowness) [nz, nx, ny] for a loss with gradient ``grad_tt_rec``
    [nsrc, nrec] on the apparent-velocity traveltimes at ``receivers`` (node
    axes from the origin 0), summed over sources: the sequential reverse-mode
    derivative of ``solve3d`` + ``vinterp``."""
    slow = _c(slow)
    src = _c(np.atleast_2d(sources))
    rec = _c(np.atleast_2d(receivers))
    g = _c(grad_tt_rec)
    nz, nx, ny = slow.shape
    out = np.empty_like(slow)
    st = lib().oracle_adjoint3d(
        _p(slow), nz, nx, ny, *map(float, gridsize), _p(src), len(src), int(nsweep), _p(rec),
        len(rec), _p(g), _p(out), int(nthreads or os.cpu_count()),
    )
    if st == 1:
        raise ValueError("source out of bound")
    return out


def solve2d(slow, gridsize, sources, nsweep=2, grad=False, nthreads=None, fast=False):
    slow = _c(slow)
    src = _c(np.atleast_2d(sources))
    nz, nx = slow.shape
    nsrc = len(src)
    tt = np.empty((nsrc, nz + 1, nx + 1))
    tg = np.empty((nsrc, nz + 1, nx + 1, 2)) if grad else np.empty(1)
    vz = np.empty(nsrc)
    nthreads = nthreads or os.cpu_count()
    st = lib(fast).oracle_fteik2d_many(
        _p(slow), nz, nx, *map(float, gridsize), _p(src), nsrc, int(nsweep), int(grad),
        _p(tt), _p(tg), _p(vz), int(nthreads),
    )
    if st == 1:
        raise ValueError("source out of bound")
    return tt, (tg if grad else None), vz


def axes(shape, gridsize, origin):
    return [origin[d] + gridsize[d] * np.arange(shape[d]) for d in range(len(shape))]


def interp(ax, v, points, fill_value=np.nan, stride=1):
    """Plain bi-/tri-linear interpolation (``_interp2d.py`` / ``_interp3d.py``).
    ``v`` may be a strided gradient component: pass the full [..][stride] array
    offset by the component via ``v[..., c]``'s base and ``stride``."""
    pts = _c(np.atleast_2d(points))
    out = np.empty(len(pts))
    ax = [_c(a) for a in ax]
    v = np.asarray(v)
    if len(ax) == 3:
        lib().oracle_interp3d(
            _p(ax[0]), len(ax[0]), _p(ax[1]), len(ax[1]), _p(ax[2]), len(ax[2]),
            ctypes.c_void_p(v.ctypes.data), stride, _p(pts), len(pts), float(fill_value), _p(out),
        )
    else:
        lib().oracle_interp2d(
            _p(ax[0]), len(ax[0]), _p(ax[1]), len(ax[1]), ctypes.c_void_p(v.ctypes.data), stride,
            _p(pts), len(pts), float(fill_value), _p(out),
        )
    return out


def vinterp(ax, tt, points, source, vzero, fill_value=np.nan):
    """Apparent-velocity traveltime interpolation (``_vinterp2d.py`` / ``_vinterp3d.py``)."""
    pts = _c(np.atleast_2d(points))
    out = np.empty(len(pts))
    ax = [_c(a) for a in ax]
    tt = _c(tt)
    src = _c(source)
    if len(ax) == 3:
        lib().oracle_vinterp3d(
            _p(ax[0]), len(ax[0]), _p(ax[1]), len(ax[1]), _p(ax[2]), len(ax[2]), _p(tt),
            _p(pts), len(pts), _p(src), float(vzero), float(fill_value), _p(out),
        )
    else:
        lib().oracle_vinterp2d(
            _p(ax[0]), len(ax[0]), _p(ax[1]), len(ax[1]), _p(tt), _p(pts), len(pts), _p(src),
            float(vzero), float(fill_value), _p(out),
        )
    return out


def raytrace(ax, ttgrad, ends, source, stepsize, max_step, honor_grid=False, fast=False):
    """Ray tracing (``_ray2d.py`` / ``_ray3d.py``). Returns a list of rays, each
    ordered source -> end point, as ``ray3d`` returns them."""
    nd = len(ax)
    ends = _c(np.atleast_2d(ends))
    n = len(ends)
    ax = [_c(a) for a in ax]
    g = _c(ttgrad)
    src = _c(source)
    rays = np.zeros((n, int(max_step), nd))
    counts = np.zeros(n, dtype=np.int32)
    status = np.zeros(n, dtype=np.int32)
    if nd == 3:
        lib(fast).oracle_ray3d(
            _p(ax[0]), len(ax[0]), _p(ax[1]), len(ax[1]), _p(ax[2]), len(ax[2]), _p(g),
            _p(ends), n, _p(src), float(stepsize), int(max_step), int(honor_grid), _p(rays),
            _p(counts), _p(status),
        )
    else:
        lib(fast).oracle_ray2d(
            _p(ax[0]), len(ax[0]), _p(ax[1]), len(ax[1]), _p(g), _p(ends), n, _p(src),
            float(stepsize), int(max_step), int(honor_grid), _p(rays), _p(counts), _p(status),
        )
    if (status == 2).any():
        raise ValueError("end point out of bound")
    if (status == 3).any():
        raise RuntimeError("maximum number of steps reached")
    return [rays[r, counts[r]::-1].copy() for r in range(n)]
