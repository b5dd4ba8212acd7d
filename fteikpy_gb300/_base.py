"""Grid base classes, mirroring fteikpy/_base.py (same names, properties,
argument meaning and errors) with device-resident storage.

A grid's values may live on the host (NumPy), on the device (a CUDA tensor) or
both; ``.grid`` always returns a NumPy array as in the reference (copied from
the device once, then cached), while the compute calls use the device copy.
Interpolation, resampling and smoothing run on the device.
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

    @property
    def tensor(self):
        """The grid values as a float64 CUDA tensor: the device memory the
        library computed them in (a solve's traveltimes, a batch's views), or
        an upload of host values made once and cached. No copy is made for
        device-resident values, so torch code can use a solve's result
        directly. No counterpart in the reference, whose grids are NumPy
        arrays (fteikpy/_base.py:22-25)."""
        return self._device_grid()

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


def _axis_table(axis, points, method):
    """Per-axis lookup of scipy's RegularGridInterpolator at ``points``
    (scipy/interpolate/_rgi.py: lower index i = searchsorted(axis, x) - 1
    clipped to [0, n - 2], normalised distance y = (x - a[i]) / (a[i+1] - a[i]);
    "nearest" takes i where y <= 0.5, else i + 1)."""
    i = np.clip(np.searchsorted(axis, points, side="left") - 1, 0, len(axis) - 2)
    y = (points - axis[i]) / (axis[i + 1] - axis[i])
    if method == "nearest":
        return np.where(y <= 0.5, i, i + 1).astype(np.int32), None, None
    return i.astype(np.int32), y, 1 - y


def _gaussian_weights(sigma, truncate=4.0):
    """scipy.ndimage.gaussian_filter1d's kernel for order 0: radius
    int(truncate * sigma + 0.5), exp(-x^2 / (2 sigma^2)) normalised to sum 1."""
    r = int(truncate * float(sigma) + 0.5)
    x = np.arange(-r, r + 1)
    phi = np.exp(-0.5 / (sigma * sigma) * x**2)
    return phi / phi.sum()


class _GridOpsMixin:
    def _resample_device(self, new_shape, method):
        """RegularGridInterpolator(axes, grid, method, bounds_error=False) at
        the tensor grid of np.linspace(axis[0], axis[-1], new_shape[d]), as
        fteikpy/_base.py:81-110,165-199 builds it, evaluated by
        ``fteik_resample``; the grid spacing follows the reference."""
        if method not in ("linear", "nearest"):
            raise ValueError(f"Method '{method}' is not defined")
        nd = self._ndim
        new_shape = tuple(int(n) for n in new_shape)
        if len(new_shape) != nd or min(new_shape) < 1:
            raise ValueError(f"new_shape must hold {nd} positive sizes")
        if min(self.shape) < 2:
            raise ValueError("resampling needs at least 2 points per dimension")
        tables = []
        for d in range(nd):
            axis = self._axis(d)
            q = np.linspace(axis[0], axis[-1], new_shape[d])
            tables.append(_axis_table(axis, q, method))
        idx = _device.to_device(np.concatenate([t[0] for t in tables]), torch.int32)
        nearest = method == "nearest"
        y = ym = None
        if not nearest:
            y = _device.to_device(np.concatenate([t[1] for t in tables]))
            ym = _device.to_device(np.concatenate([t[2] for t in tables]))
        v = self._device_grid().contiguous()
        out = torch.empty(new_shape, dtype=torch.float64, device=v.device)
        dims = np.ascontiguousarray(self.shape, dtype=np.int32)
        odims = np.ascontiguousarray(new_shape, dtype=np.int32)
        rc = _lib.load().fteik_resample(
            nd, int(nearest), _device.ptr(v), _device.host_ptr(dims), _device.host_ptr(odims),
            _device.ptr(idx), _device.ptr(y), _device.ptr(ym), _device.ptr(out),
            _device.stream(),
        )
        _lib.check(rc, "resample")
        old_shape = self.shape
        self._grid = out
        self._gridsize = tuple(a * b / c for a, b, c in zip(self.gridsize, old_shape, new_shape))

    def _smooth_device(self, sigma):
        """gaussian_filter(grid, sigma / gridsize) (fteikpy/_base.py:112-123,
        201-212): one 1D correlation per axis whose sigma exceeds 1e-15, in
        axis order, mode 'reflect', truncate 4, by ``fteik_correlate1d``."""
        nd = self._ndim
        sigma = np.full(nd, sigma) if np.ndim(sigma) == 0 else np.asarray(sigma)
        sig = np.asarray(sigma, dtype=np.float64) / np.asarray(self._gridsize)
        lib = _lib.load()
        cur = self._device_grid().contiguous()
        dims = np.ascontiguousarray(cur.shape, dtype=np.int32)
        for d in range(nd):
            if not sig[d] > 1e-15:
                continue
            w = _device.to_device(_gaussian_weights(sig[d]))
            out = torch.empty_like(cur)
            rc = lib.fteik_correlate1d(
                nd, _device.ptr(cur), _device.host_ptr(dims), d, _device.ptr(w), w.numel(),
                _device.ptr(out), _device.stream(),
            )
            _lib.check(rc, "smooth")
            cur = out
        self._grid = cur.clone() if cur is self._dev else cur


class BaseGrid2D(BaseGrid, _GridOpsMixin):
    _ndim = 2

    def __call__(self, points, fill_value=np.nan):
        """Bilinear interpolation (fteikpy/_base.py:56-79)."""
        return self._interp_device(points, fill_value)

    def resample(self, new_shape, method="linear"):
        """Resample grid (fteikpy/_base.py:81-110), on the device."""
        self._resample_device(new_shape, method)

    def smooth(self, sigma):
        """Smooth grid (fteikpy/_base.py:112-123), on the device."""
        self._smooth_device(sigma)

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


class BaseGrid3D(BaseGrid, _GridOpsMixin):
    _ndim = 3

    def __call__(self, points, fill_value=np.nan):
        """Trilinear interpolation (fteikpy/_base.py:139-163)."""
        return self._interp_device(points, fill_value)

    def resample(self, new_shape, method="linear"):
        """Resample grid (fteikpy/_base.py:165-199), on the device."""
        self._resample_device(new_shape, method)

    def smooth(self, sigma):
        """Smooth grid (fteikpy/_base.py:201-212), on the device."""
        self._smooth_device(sigma)

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
