"""Grid base classes, mirroring fteikpy/_base.py (same names, properties,
argument meaning and errors) with device-resident storage.

A grid's values may live on the host (NumPy), on the device (a CUDA tensor) or
both; ``.grid`` always returns a NumPy array as in the reference (copied from
the device once, then cached), while the compute calls use the device copy.
"""

from abc import ABC

import numpy as np
import torch

from . import _device, _lib


class BaseGrid(ABC):
    def __init__(self, grid, gridsize, origin, **kwargs):
        """Base grid class (fteikpy/_base.py:10-16)."""
        super().__init__(**kwargs)
        self._set_values(grid)
        self._gridsize = tuple(float(x) for x in gridsize)
        self._origin = np.asarray(origin, dtype=np.float64)
        self._axes_cache = None

    # -- storage -------------------------------------------------------------
    def _set_values(self, grid):
        if isinstance(grid, torch.Tensor):
            self._dev = grid if grid.dtype == torch.float64 else grid.to(torch.float64)
            self._host = None
        else:
            self._host = np.asarray(grid, dtype=np.float64)
            self._dev = None
        self._slow_cache = None

    @property
    def _grid(self):
        if self._host is None:
            self._host = self._dev.detach().cpu().numpy()
        return self._host

    @_grid.setter
    def _grid(self, value):
        self._set_values(value)
        self._axes_cache = None

    def _device_grid(self):
        """Grid values as a CUDA tensor (uploaded once, then cached)."""
        if self._dev is None or self._dev.device.type != "cuda":
            self._dev = _device.to_device(self._host)
        return self._dev

    def _device_axes(self):
        if self._axes_cache is None:
            self._axes_cache = [_device.to_device(a) for a in self._axes()]
        return self._axes_cache

    # -- reference API -----------------------------------------------------------
    def __getitem__(self, islice):
        """Slice grid."""
        return self._grid[islice]

    @property
    def grid(self):
        """Return grid."""
        return self._grid

    @property
    def gridsize(self):
        """Return grid size."""
        return self._gridsize

    @property
    def origin(self):
        """Return grid origin coordinates."""
        return self._origin

    @property
    def shape(self):
        """Return grid shape."""
        return tuple(self._host.shape if self._host is not None else self._dev.shape)

    @property
    def size(self):
        """Return grid size."""
        return int(np.prod(self.shape))

    @property
    def ndim(self):
        """Return grid number of dimensions."""
        return len(self.shape)

    def _axis(self, d):
        return self._origin[d] + self._gridsize[d] * np.arange(self.shape[d])

    def _interp_device(self, points, fill_value):
        """Bi-/tri-linear interpolation on the device (fteikpy/_interp/_interp*d.py)."""
        nd = self._ndim
        pts = np.asarray(points, dtype=np.float64)
        single = pts.ndim == 1
        pts2 = np.ascontiguousarray(np.atleast_2d(pts))
        if pts2.shape[-1] != nd:
            raise ValueError(f"points must have {nd} coordinates")
        lib = _lib.load()
        v = self._device_grid()
        vs = 1
        if not v.is_contiguous():
            # a gradient component: a strided view of a [..., ndim] array
            st = v.stride()
            sh = v.shape
            inner = st[-1]
            expect = [inner]
            for n in reversed(sh[1:]):
                expect.insert(0, expect[0] * n)
            if list(st) == expect:
                vs = inner
            else:
                v = v.contiguous()
        ax = self._device_axes()
        q = _device.to_device(pts2)
        out = torch.empty(len(pts2), dtype=torch.float64, device=q.device)
        if nd == 3:
            rc = lib.fteik_interp3d(
                _device.ptr(ax[0]), len(ax[0]), _device.ptr(ax[1]), len(ax[1]),
                _device.ptr(ax[2]), len(ax[2]), _device.ptr(v), vs, _device.ptr(q), len(pts2),
                float(fill_value), _device.ptr(out), _device.stream(),
            )
        else:
            rc = lib.fteik_interp2d(
                _device.ptr(ax[0]), len(ax[0]), _device.ptr(ax[1]), len(ax[1]), _device.ptr(v),
                vs, _device.ptr(q), len(pts2), float(fill_value), _device.ptr(out),
                _device.stream(),
            )
        _lib.check(rc, "interp")
        res = out.cpu().numpy()
        return float(res[0]) if single else res


class BaseGrid2D(BaseGrid):
    _ndim = 2

    def __call__(self, points, fill_value=np.nan):
        """Bilinear interpolation (fteikpy/_base.py:56-79)."""
        return self._interp_device(points, fill_value)

    def resample(self, new_shape, method="linear"):
        """Resample grid (fteikpy/_base.py:81-110; model preparation, done with
        SciPy on the host exactly as the reference does)."""
        from scipy.interpolate import RegularGridInterpolator

        zaxis = self.zaxis
        xaxis = self.xaxis
        Z, X = np.meshgrid(
            np.linspace(zaxis[0], zaxis[-1], new_shape[0]),
            np.linspace(xaxis[0], xaxis[-1], new_shape[1]),
            indexing="ij",
        )
        fn = RegularGridInterpolator(
            points=(zaxis, xaxis), values=self._grid, method=method, bounds_error=False
        )
        self._grid = fn([[z, x] for z, x in zip(Z.ravel(), X.ravel())]).reshape(new_shape)
        self._gridsize = tuple(
            a * b / c for a, b, c in zip(self.gridsize, self.shape, new_shape)
        )

    def smooth(self, sigma):
        """Smooth grid (fteikpy/_base.py:112-123; SciPy on the host)."""
        from scipy.ndimage import gaussian_filter

        sigma = np.full(2, sigma) if np.ndim(sigma) == 0 else np.asarray(sigma)
        self._grid = gaussian_filter(self._grid, sigma / self._gridsize)

    def _axes(self):
        return [self.zaxis, self.xaxis]

    @property
    def zaxis(self):
        """Return grid Z axis."""
        return self._axis(0)

    @property
    def xaxis(self):
        """Return grid X axis."""
        return self._axis(1)


class BaseGrid3D(BaseGrid):
    _ndim = 3

    def __call__(self, points, fill_value=np.nan):
        """Trilinear interpolation (fteikpy/_base.py:139-163)."""
        return self._interp_device(points, fill_value)

    def resample(self, new_shape, method="linear"):
        """Resample grid (fteikpy/_base.py:165-199; SciPy on the host)."""
        from scipy.interpolate import RegularGridInterpolator

        zaxis = self.zaxis
        xaxis = self.xaxis
        yaxis = self.yaxis
        Z, X, Y = np.meshgrid(
            np.linspace(zaxis[0], zaxis[-1], new_shape[0]),
            np.linspace(xaxis[0], xaxis[-1], new_shape[1]),
            np.linspace(yaxis[0], yaxis[-1], new_shape[2]),
            indexing="ij",
        )
        fn = RegularGridInterpolator(
            points=(zaxis, xaxis, yaxis), values=self._grid, method=method, bounds_error=False
        )
        self._grid = fn(
            [[z, x, y] for z, x, y in zip(Z.ravel(), X.ravel(), Y.ravel())]
        ).reshape(new_shape)
        self._gridsize = tuple(
            a * b / c for a, b, c in zip(self.gridsize, self.shape, new_shape)
        )

    def smooth(self, sigma):
        """Smooth grid (fteikpy/_base.py:201-212; SciPy on the host)."""
        from scipy.ndimage import gaussian_filter

        sigma = np.full(3, sigma) if np.ndim(sigma) == 0 else np.asarray(sigma)
        self._grid = gaussian_filter(self._grid, sigma / self._gridsize)

    def _axes(self):
        return [self.zaxis, self.xaxis, self.yaxis]

    @property
    def zaxis(self):
        """Return grid Z axis."""
        return self._axis(0)

    @property
    def xaxis(self):
        """Return grid X axis."""
        return self._axis(1)

    @property
    def yaxis(self):
        """Return grid Y axis."""
        return self._axis(2)


class BaseTraveltime(ABC):
    def __init__(self, source, gradient, vzero, **kwargs):
        """Traveltime base class (fteikpy/_base.py:230-241)."""
        super().__init__(**kwargs)
        self._source = source
        self._gradient = gradient
        self._vzero = vzero

    @property
    def source(self):
        """Return source coordinates."""
        return self._source
