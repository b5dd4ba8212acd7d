"""Result grids, mirroring fteikpy/_grid.py: ``Grid2D/3D`` and
``TraveltimeGrid2D/3D`` with ``__call__`` (apparent-velocity interpolation),
``raytrace`` and ``gradient``, all computed by the library's CUDA kernels.
"""

import numpy as np
import torch

from . import _device, _lib
from ._base import BaseGrid2D, BaseGrid3D, BaseTraveltime


class Grid2D(BaseGrid2D):
    def __init__(self, *args, **kwargs):
        """2D grid class (fteikpy/_grid.py:8-23)."""
        super().__init__(*args, **kwargs)


class Grid3D(BaseGrid3D):
    def __init__(self, *args, **kwargs):
        """3D grid class (fteikpy/_grid.py:26-41)."""
        super().__init__(*args, **kwargs)


def _as_gradient(gradient):
    if gradient is None or isinstance(gradient, torch.Tensor):
        return gradient
    return np.asarray(gradient, dtype=np.float64)


class _TraveltimeMixin:
    """Device implementations shared by the 2D and 3D traveltime grids."""

    def _device_gradient(self):
        g = self._gradient
        if isinstance(g, np.ndarray):
            g = _device.to_device(g)
            self._gradient = g
        return g.contiguous()

    @property
    def gradient_tensor(self):
        """The traveltime gradient, [..., ndim] float64 on the device: the
        memory the solve wrote it to (no copy). No counterpart in the
        reference, whose gradient grids are NumPy arrays (fteikpy/_grid.py:
        148-158,268-278); raises the reference's error when the solve returned
        no gradient."""
        if self._gradient is None:
            raise ValueError(
                "no gradient grid, use option `return_gradient` to return gradient grids"
            )
        return self._device_gradient()

    def _device_source(self):
        """[source coordinates..., vzero] as a CUDA tensor, uploaded once (the
        per-call interpolation and ray tracing read them on the device)."""
        c = getattr(self, "_source_cache", None)
        if c is None:
            host = np.append(np.asarray(self._source, dtype=np.float64).reshape(-1),
                             float(self._vzero))
            c = _device.to_device(host)
            self._source_cache = c
        return c

    def _vinterp(self, points, fill_value):
        nd = self._ndim
        pts = np.asarray(points, dtype=np.float64)
        single = pts.ndim == 1
        pts2 = np.ascontiguousarray(np.atleast_2d(pts))
        lib = _lib.load()
        tt = self._device_grid().contiguous()
        ax = self._device_axes()
        q = _device.to_device(pts2)
        sv = self._device_source()
        src, vz = sv[:nd], sv[nd:]
        out = torch.empty(len(pts2), dtype=torch.float64, device=q.device)
        if nd == 3:
            rc = lib.fteik_vinterp3d(
                _device.ptr(ax[0]), len(ax[0]), _device.ptr(ax[1]), len(ax[1]),
                _device.ptr(ax[2]), len(ax[2]), _device.ptr(tt), 0, None, _device.ptr(q),
                len(pts2), _device.ptr(src), _device.ptr(vz), float(fill_value),
                _device.ptr(out), _device.stream(),
            )
        else:
            rc = lib.fteik_vinterp2d(
                _device.ptr(ax[0]), len(ax[0]), _device.ptr(ax[1]), len(ax[1]), _device.ptr(tt),
                0, None, _device.ptr(q), len(pts2), _device.ptr(src), _device.ptr(vz),
                float(fill_value), _device.ptr(out), _device.stream(),
            )
        _lib.check(rc, "vinterp")
        res = out.cpu().numpy()
        return float(res[0]) if single else res

    def _raytrace(self, points, stepsize, max_step, honor_grid):
        nd = self._ndim
        if self._gradient is None:  # the reference's error (fteikpy/_grid.py:270-273)
            raise ValueError(
                "no gradient grid, use option `return_gradient` to return gradient grids"
            )
        if honor_grid or not stepsize:
            stepsize = np.min(self._gridsize)
        if not max_step:
            max_dist = 2.0 * sum((n * d) ** 2 for n, d in zip(self.shape, self._gridsize)) ** 0.5
            max_step = int(max_dist / stepsize)
        pts = np.asarray(points, dtype=np.float64)
        rays = trace_rays(
            nd, self._device_axes(), self._device_gradient(), None, pts.reshape(-1, nd),
            self._device_source()[:nd].reshape(1, nd), float(stepsize), int(max_step),
            bool(honor_grid),
        )
        return rays[0] if pts.ndim == 1 else rays


def trace_rays_device(nd, axes, ttgrad, grid_index, ends, sources, stepsize, max_step,
                      honor_grid, grad_stride=0):
    """Trace rays on the device; return (packed rays, per-ray lengths) as device
    tensors, each ray source first (the order ``ray3d`` returns).

    ``ttgrad`` is a contiguous device tensor holding one gradient grid, or a
    batch of them ``grad_stride`` elements apart selected per ray by
    ``grid_index`` (device int32, or None); ``sources`` holds one absolute
    source per grid. Raises the reference's exceptions
    (fteikpy/_fteik/_ray3d.py:33-34,115-116).
    """
    lib = _lib.load()
    dev = _device.device()
    rays, counts, status, n = _launch_rays(
        lib, nd, axes, ttgrad, grid_index, ends, sources, stepsize, max_step, honor_grid,
        grad_stride,
    )
    if n == 0:
        return (torch.empty((0, nd), dtype=torch.float64, device=dev),
                torch.zeros(0, dtype=torch.int64, device=dev))
    lengths = counts.to(torch.int64) + 1
    packed, _ = _pack_rays(lib, nd, rays, n, max_step, counts, status, lengths)
    return packed, lengths


def _launch_rays(lib, nd, axes, ttgrad, grid_index, ends, sources, stepsize, max_step,
                 honor_grid, grad_stride):
    """Launch the ray kernel; return (rays, counts, status, nrays) on the device."""
    if max_step < 2:
        raise ValueError("max_step must be at least 2")
    dev = _device.device()
    e = ends if isinstance(ends, torch.Tensor) else _device.to_device(np.ascontiguousarray(ends, dtype=np.float64))
    n = e.shape[0]
    if n == 0:
        return None, None, None, 0
    src = sources if isinstance(sources, torch.Tensor) else _device.to_device(np.ascontiguousarray(sources, dtype=np.float64))
    rays = torch.empty((n, max_step, nd), dtype=torch.float64, device=dev)
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    status = torch.empty(n, dtype=torch.int32, device=dev)
    gi = _device.ptr(grid_index) if grid_index is not None else None
    if nd == 3:
        rc = lib.fteik_ray3d(
            _device.ptr(axes[0]), len(axes[0]), _device.ptr(axes[1]), len(axes[1]),
            _device.ptr(axes[2]), len(axes[2]), _device.ptr(ttgrad), int(grad_stride), gi,
            _device.ptr(e), n, _device.ptr(src), stepsize, max_step, int(honor_grid),
            _device.ptr(rays), _device.ptr(counts), _device.ptr(status), _device.stream(),
        )
    else:
        rc = lib.fteik_ray2d(
            _device.ptr(axes[0]), len(axes[0]), _device.ptr(axes[1]), len(axes[1]),
            _device.ptr(ttgrad), int(grad_stride), gi, _device.ptr(e), n, _device.ptr(src),
            stepsize, max_step, int(honor_grid), _device.ptr(rays), _device.ptr(counts),
            _device.ptr(status), _device.stream(),
        )
    _lib.check(rc, "raytrace")
    return rays, counts, status, n


def _pack_rays(lib, nd, rays, n, max_step, counts, status, lengths):
    """Check the per-ray status and pack the rays source first; one host
    round trip brings back the worst status, the total length and the
    per-ray lengths. Returns (packed device rays, host lengths)."""
    dev = rays.device
    offsets = torch.cumsum(lengths, 0) - lengths
    info = torch.cat([status.max().to(torch.int64).reshape(1), lengths]).cpu().numpy()
    worst, host_lengths = int(info[0]), info[1:]
    if worst != _lib.OK:
        st = status.cpu().numpy()
        if (st == _lib.END_POINT_OUT_OF_BOUND).any():
            raise ValueError("end point out of bound")
        raise RuntimeError("maximum number of steps reached")
    packed = torch.empty((int(host_lengths.sum()), nd), dtype=torch.float64, device=dev)
    rc = lib.fteik_ray_pack(
        nd, _device.ptr(rays), n, max_step, _device.ptr(counts), _device.ptr(offsets),
        _device.ptr(packed), _device.stream(),
    )
    _lib.check(rc, "raytrace")
    return packed, host_lengths


def trace_rays(nd, axes, ttgrad, grid_index, ends, sources, stepsize, max_step, honor_grid,
               grad_stride=0):
    """``trace_rays_device`` followed by the copy to the host: a list of NumPy
    rays, as ``ray3d`` / ``ray2d`` return for several end points."""
    lib = _lib.load()
    rays, counts, status, n = _launch_rays(
        lib, nd, axes, ttgrad, grid_index, ends, sources, stepsize, max_step, honor_grid,
        grad_stride,
    )
    if n == 0:
        return []
    lengths = counts.to(torch.int64) + 1
    packed, host_lengths = _pack_rays(lib, nd, rays, n, max_step, counts, status, lengths)
    flat = packed.cpu().numpy()
    ends = np.cumsum(host_lengths).tolist()
    # views into one host array, as np.split returns them (slicing is faster)
    return [flat[b - n:b] for b, n in zip(ends, host_lengths.tolist())]


class TraveltimeGrid2D(BaseGrid2D, BaseTraveltime, _TraveltimeMixin):
    def __init__(self, grid, gridsize, origin, source, gradient, vzero):
        """2D traveltime grid class (fteikpy/_grid.py:44-74)."""
        super().__init__(
            grid=grid,
            gridsize=gridsize,
            origin=np.asarray(origin, dtype=np.float64),
            source=np.asarray(source, dtype=np.float64),
            gradient=_as_gradient(gradient),
            vzero=vzero,
        )

    def __call__(self, points, fill_value=np.nan):
        """Bilinear apparent velocity interpolation (fteikpy/_grid.py:76-101)."""
        return self._vinterp(points, fill_value)

    def raytrace(self, points, stepsize=None, max_step=None, honor_grid=False):
        """2D a posteriori ray-tracing (fteikpy/_grid.py:103-145)."""
        return self._raytrace(points, stepsize, max_step, honor_grid)

    @property
    def gradient(self):
        """Return Z and X gradient grids as a list of :class:`Grid2D`."""
        if self._gradient is None:
            raise ValueError(
                "no gradient grid, use option `return_gradient` to return gradient grids"
            )
        return [Grid2D(self._gradient[:, :, i], self._gridsize, self._origin) for i in range(2)]


class TraveltimeGrid3D(BaseGrid3D, BaseTraveltime, _TraveltimeMixin):
    def __init__(self, grid, gridsize, origin, source, gradient, vzero):
        """3D traveltime grid class (fteikpy/_grid.py:161-191)."""
        super().__init__(
            grid=grid,
            gridsize=gridsize,
            origin=np.asarray(origin, dtype=np.float64),
            source=np.asarray(source, dtype=np.float64),
            gradient=_as_gradient(gradient),
            vzero=vzero,
        )

    def __call__(self, points, fill_value=np.nan):
        """Trilinear apparent velocity interpolation (fteikpy/_grid.py:193-219)."""
        return self._vinterp(points, fill_value)

    def raytrace(self, points, stepsize=None, max_step=None, honor_grid=False):
        """3D a posteriori ray-tracing (fteikpy/_grid.py:221-265)."""
        return self._raytrace(points, stepsize, max_step, honor_grid)

    @property
    def gradient(self):
        """Return Z, X and Y gradient grids as a list of :class:`Grid3D`."""
        if self._gradient is None:
            raise ValueError(
                "no gradient grid, use option `return_gradient` to return gradient grids"
            )
        return [
            Grid3D(self._gradient[:, :, :, i], self._gridsize, self._origin) for i in range(3)
        ]
