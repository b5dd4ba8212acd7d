"""Eikonal solvers, mirroring fteikpy/_solver.py: ``Eikonal2D`` / ``Eikonal3D``
with ``solve(sources, nsweep=2, return_gradient=False)``.

The solve runs on the GPU through ``fteik2d_solve`` / ``fteik3d_solve`` of the C
ABI. Results stay on the device: every returned ``TraveltimeGrid*`` wraps a
view of one batched device tensor, and ``.grid`` copies it to the host only
when read.
"""

import ctypes

import numpy as np
import torch

from . import _device, _lib
from ._base import BaseGrid2D, BaseGrid3D
from ._grid import TraveltimeGrid2D, TraveltimeGrid3D

# Polls of one device-side dependency wait before a solve gives up with an
# error instead of waiting forever (tests lower it to exercise the error path).
SPIN_LIMIT = 1 << 25


class _SolverMixin:
    def _device_slowness(self):
        """1.0 / velocity on the device (fteikpy/_solver.py:49,121), cached."""
        if self._slow_cache is None:
            self._slow_cache = _device.slowness(self._device_grid())
        return self._slow_cache

    def _prepare_sources(self, sources):
        sources = np.asarray(sources, dtype=np.float64)
        rel = sources - self._origin
        if rel.ndim not in (1, 2) or rel.shape[-1] != self._ndim:
            raise ValueError(f"sources must have shape ({self._ndim},) or (n, {self._ndim})")
        return sources, rel

    def _wrap(self, cls, sources, rel, tt, ttgrad, vzero, return_gradient):
        vz = vzero.cpu().numpy()
        if rel.ndim == 2:
            return [
                cls(
                    grid=tt[i],
                    gridsize=self._gridsize,
                    origin=self._origin,
                    source=sources[i],
                    gradient=ttgrad[i] if return_gradient else None,
                    vzero=float(vz[i]),
                )
                for i in range(len(rel))
            ]
        return cls(
            grid=tt[0],
            gridsize=self._gridsize,
            origin=self._origin,
            source=sources,
            gradient=ttgrad[0] if return_gradient else None,
            vzero=float(vz[0]),
        )


class Eikonal2D(BaseGrid2D, _SolverMixin):
    def __init__(self, grid, gridsize, origin=None):
        """2D Eikonal solver (fteikpy/_solver.py:8-27).

        Parameters
        ----------
        grid : array_like or torch.Tensor
            Velocity model array (a CUDA tensor is used in place).
        gridsize : array_like
            Grid size (dz, dx).
        origin : array_like or None, optional, default None
            Grid origin coordinates.
        """
        super().__init__(
            grid=grid,
            gridsize=gridsize,
            origin=origin if origin is not None else np.zeros(2, dtype=np.float64),
        )

    def solve(self, sources, nsweep=2, return_gradient=False):
        """Solve Eikonal for given sources (fteikpy/_solver.py:29-77).

        Returns a :class:`TraveltimeGrid2D`, or a list of them when ``sources``
        is a list of source coordinates.
        """
        sources, rel = self._prepare_sources(sources)
        src = np.ascontiguousarray(np.atleast_2d(rel))
        nsrc = len(src)
        nz, nx = self.shape
        grad = bool(return_gradient)
        slow = self._device_slowness()
        dev = slow.device
        tt = torch.empty((nsrc, nz + 1, nx + 1), dtype=torch.float64, device=dev)
        ttgrad = (
            torch.empty((nsrc, nz + 1, nx + 1, 2), dtype=torch.float64, device=dev)
            if grad
            else None
        )
        vzero = torch.empty(nsrc, dtype=torch.float64, device=dev)
        lib = _lib.load()
        nbytes = lib.fteik2d_workspace_bytes(nz, nx, nsrc, int(grad))
        ws = _device.workspace("solve2d", nbytes)
        rc = lib.fteik2d_solve(
            _device.ptr(slow), nz, nx, *self._gridsize, _device.host_ptr(src), nsrc,
            max(int(nsweep), 0), int(grad), _device.ptr(tt), _device.ptr(ttgrad),
            _device.ptr(vzero), _device.ptr(ws), ws.numel(), _device.stream(),
        )
        _lib.check(rc, "Eikonal2D.solve")
        return self._wrap(TraveltimeGrid2D, sources, rel, tt, ttgrad, vzero, grad)


class Eikonal3D(BaseGrid3D, _SolverMixin):
    def __init__(self, grid, gridsize, origin=None):
        """3D Eikonal solver (fteikpy/_solver.py:80-99).

        Parameters
        ----------
        grid : array_like or torch.Tensor
            Velocity model array (a CUDA tensor is used in place).
        gridsize : array_like
            Grid size (dz, dx, dy).
        origin : array_like or None, optional, default None
            Grid origin coordinates.
        """
        super().__init__(
            grid=grid,
            gridsize=gridsize,
            origin=origin if origin is not None else np.zeros(3, dtype=np.float64),
        )

    def solve(self, sources, nsweep=2, return_gradient=False):
        """Solve Eikonal for given sources (fteikpy/_solver.py:101-149).

        Every source is solved by the same persistent kernel launch. Returns a
        :class:`TraveltimeGrid3D`, or a list of them when ``sources`` is a list
        of source coordinates.
        """
        sources, rel = self._prepare_sources(sources)
        src = np.ascontiguousarray(np.atleast_2d(rel))
        tt, ttgrad, vzero = solve3d_device(
            self._device_slowness(), self._gridsize, src, nsweep, return_gradient
        )
        return self._wrap(TraveltimeGrid3D, sources, rel, tt, ttgrad, vzero, return_gradient)


def solve3d_device(slow, gridsize, src, nsweep=2, return_gradient=False, spin_limit=None,
                   workspace=None, record=False):
    """Batched 3D solve on device tensors: ``slow`` [nz, nx, ny] (CUDA, float64),
    ``src`` [nsrc, 3] host coordinates relative to the grid origin.
    Returns device tensors (tt, ttgrad or None, vzero).

    ``record=True`` keeps the branch record in ``workspace`` (a uint8 CUDA
    tensor of at least ``fteik3d_workspace_bytes`` bytes) for the adjoint."""
    src = np.ascontiguousarray(np.atleast_2d(src), dtype=np.float64)
    nsrc = len(src)
    nz, nx, ny = slow.shape
    grad = 1 if return_gradient else (2 if record else 0)
    dev = slow.device
    tt = torch.empty((nsrc, nz + 1, nx + 1, ny + 1), dtype=torch.float64, device=dev)
    ttgrad = (
        torch.empty((nsrc, nz + 1, nx + 1, ny + 1, 3), dtype=torch.float64, device=dev)
        if grad == 1
        else None
    )
    vzero = torch.empty(nsrc, dtype=torch.float64, device=dev)
    lib = _lib.load()
    nbytes = lib.fteik3d_workspace_bytes(nz, nx, ny, nsrc, int(grad))
    ws = workspace if workspace is not None else _device.workspace("solve3d", nbytes)
    if ws.numel() < nbytes:
        raise ValueError("workspace too small")
    rc = lib.fteik3d_solve(
        _device.ptr(slow), nz, nx, ny, *[float(g) for g in gridsize], _device.host_ptr(src),
        nsrc, max(int(nsweep), 0), int(grad), _device.ptr(tt), _device.ptr(ttgrad),
        _device.ptr(vzero), _device.ptr(ws), ws.numel(),
        int(spin_limit if spin_limit is not None else SPIN_LIMIT), _device.stream(),
    )
    _lib.check(rc, "Eikonal3D.solve")
    return tt, ttgrad, vzero


def _batch_arguments(solvers, sources, return_gradient):
    """Host and device arguments of fteik3d_solve_batch for Eikonal3D solvers."""
    if len(solvers) != len(sources) or not solvers:
        raise ValueError("solvers and sources must be non-empty lists of the same length")
    grad = bool(return_gradient)
    slows, dims, spacing, rels, given, tts, grads = [], [], [], [], [], [], []
    for eik, src in zip(solvers, sources):
        if not isinstance(eik, Eikonal3D):
            raise TypeError("solve_batch takes Eikonal3D solvers")
        src_abs, rel = eik._prepare_sources(src)
        slow = eik._device_slowness()
        nz, nx, ny = slow.shape
        rel2 = np.ascontiguousarray(np.atleast_2d(rel), dtype=np.float64)
        tt = torch.empty((len(rel2), nz + 1, nx + 1, ny + 1), dtype=torch.float64,
                         device=slow.device)
        g = (torch.empty((len(rel2), nz + 1, nx + 1, ny + 1, 3), dtype=torch.float64,
                         device=slow.device) if grad else None)
        slows.append(slow)
        dims.append((nz, nx, ny))
        spacing.append(tuple(float(h) for h in eik._gridsize))
        rels.append(rel2)
        given.append((src_abs, rel))
        tts.append(tt)
        grads.append(g)
    n = len(solvers)
    P = ctypes.c_void_p * n
    args = dict(
        n=n,
        slow=P(*[_device.ptr(x) for x in slows]),
        dims=np.ascontiguousarray(dims, dtype=np.int32),
        spacing=np.ascontiguousarray(spacing, dtype=np.float64),
        sources=np.ascontiguousarray(np.concatenate(rels), dtype=np.float64),
        nsrc=np.ascontiguousarray([len(r) for r in rels], dtype=np.int32),
        tt=P(*[_device.ptr(x) for x in tts]),
        ttgrad=P(*[_device.ptr(x) for x in grads]) if grad else None,
        vzero=torch.empty(sum(len(r) for r in rels), dtype=torch.float64,
                          device=slows[0].device),
        grad=int(grad),
    )
    return args, given, tts, grads


def _batch_workspace(lib, a):
    nbytes = lib.fteik3d_batch_workspace_bytes(
        a["n"], _device.host_ptr(a["dims"]), _device.host_ptr(a["nsrc"]), a["grad"]
    )
    if nbytes == 0:
        raise ValueError("invalid model sizes or source counts")
    return _device.workspace("batch3d", nbytes)


def solve_batch(solvers, sources, nsweep=2, return_gradient=False):
    """Solve several 3D models, each with its own sources, in one GPU launch.

    No counterpart in the reference, where each model is solved by its own
    ``Eikonal3D.solve`` (fteikpy/_solver.py:101-149); the results are the same.

    Parameters
    ----------
    solvers : list of Eikonal3D
        Models of any sizes and grid spacings.
    sources : list of array_like
        Per solver, the source coordinates as ``Eikonal3D.solve`` takes them.
    nsweep, return_gradient : as ``Eikonal3D.solve``.

    Returns
    -------
    list, per solver, of what ``Eikonal3D.solve`` would return.
    """
    lib = _lib.load()
    a, given, tts, grads = _batch_arguments(solvers, sources, return_gradient)
    ws = _batch_workspace(lib, a)
    rc = lib.fteik3d_solve_batch(
        a["n"], a["slow"], _device.host_ptr(a["dims"]), _device.host_ptr(a["spacing"]),
        _device.host_ptr(a["sources"]), _device.host_ptr(a["nsrc"]), max(int(nsweep), 0),
        a["grad"], a["tt"], a["ttgrad"], _device.ptr(a["vzero"]), _device.ptr(ws), ws.numel(),
        int(SPIN_LIMIT), _device.stream(),
    )
    _lib.check(rc, "solve_batch")
    out, off = [], 0
    for eik, (src_abs, rel), tt, g in zip(solvers, given, tts, grads):
        n = tt.shape[0]
        out.append(eik._wrap(TraveltimeGrid3D, src_abs, rel, tt, g, a["vzero"][off:off + n],
                             bool(return_gradient)))
        off += n
    return out


def autotune(solvers, sources, return_gradient=False):
    """Measure the fastest launch shape of the 3D sweep kernel for a problem
    and use it for every later solve of the same signature (cell counts,
    source counts, gradients) in this process.

    ``solvers`` is one Eikonal3D (``sources`` as its ``solve`` takes them) or a
    list of them (``sources`` a list, as ``solve_batch`` takes them). Returns
    {"pencil": w, "chunk": c, "coef": f, "team": m, "ms": t}: pencil width
    along x, steps between progress publications, coefficient source (1
    arrays, 0 cells), whether blocks of 4 sources step together with
    compacted operators, and the sweep kernel's time for one sweep per
    direction.
    """
    lib = _lib.load()
    shape = (ctypes.c_int * 4)()
    ms = ctypes.c_float()
    if isinstance(solvers, Eikonal3D):
        src = np.ascontiguousarray(np.atleast_2d(solvers._prepare_sources(sources)[1]))
        slow = solvers._device_slowness()
        nz, nx, ny = slow.shape
        grad = 1 if return_gradient else 0
        tt = torch.empty((len(src), nz + 1, nx + 1, ny + 1), dtype=torch.float64,
                         device=slow.device)
        g = (torch.empty((len(src), nz + 1, nx + 1, ny + 1, 3), dtype=torch.float64,
                         device=slow.device) if grad else None)
        vz = torch.empty(len(src), dtype=torch.float64, device=slow.device)
        ws = _device.workspace("solve3d", lib.fteik3d_workspace_bytes(nz, nx, ny, len(src), grad))
        rc = lib.fteik3d_autotune(
            _device.ptr(slow), nz, nx, ny, *solvers._gridsize, _device.host_ptr(src), len(src),
            grad, _device.ptr(tt), _device.ptr(g), _device.ptr(vz), _device.ptr(ws), ws.numel(),
            int(SPIN_LIMIT), shape, ctypes.byref(ms), _device.stream(),
        )
    else:
        a, _, _, _ = _batch_arguments(list(solvers), list(sources), return_gradient)
        ws = _batch_workspace(lib, a)
        rc = lib.fteik3d_batch_autotune(
            a["n"], a["slow"], _device.host_ptr(a["dims"]), _device.host_ptr(a["spacing"]),
            _device.host_ptr(a["sources"]), _device.host_ptr(a["nsrc"]), a["grad"], a["tt"],
            a["ttgrad"], _device.ptr(a["vzero"]), _device.ptr(ws), ws.numel(), int(SPIN_LIMIT),
            shape, ctypes.byref(ms), _device.stream(),
        )
    _lib.check(rc, "autotune")
    return {"pencil": shape[0], "chunk": shape[1], "coef": shape[2], "team": shape[3],
            "ms": float(ms.value)}
