"""Eikonal solvers, mirroring fteikpy/_solver.py: ``Eikonal2D`` / ``Eikonal3D``
with ``solve(sources, nsweep=2, return_gradient=False)``.

The solve runs on the GPU through ``fteik2d_solve`` / ``fteik3d_solve`` of the C
ABI. Results stay on the device: every returned ``TraveltimeGrid*`` wraps a
view of one batched device tensor, and ``.grid`` copies it to the host only
when read.
"""

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
