"""Shared test helpers: error metrics and the reference's own known answers."""

import numpy as np


def max_rel(a, b):
    """Largest |a - b| / |b| over the arrays (|a - b| where b == 0); NaNs must match."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    na, nb = np.isnan(a), np.isnan(b)
    assert np.array_equal(na, nb), "NaN pattern differs"
    a, b = a[~na], b[~nb]
    if a.size == 0:
        return 0.0
    d = np.abs(a - b)
    return float(np.max(np.where(b != 0.0, d / np.abs(np.where(b != 0.0, b, 1.0)), d)))


def ray_lengths(rays):
    return np.array([len(r) for r in rays])


def model_axes(shape, gridsize, origin):
    return [origin[d] + gridsize[d] * np.arange(shape[d]) for d in range(len(shape))]


def default_max_step(shape, gridsize, stepsize):
    """``TraveltimeGrid*.raytrace`` default (``fteikpy/_grid.py:129-133,247-251``)."""
    max_dist = 2.0 * sum((n * d) ** 2 for n, d in zip(shape, gridsize)) ** 0.5
    return int(max_dist / stepsize)


# Known answers from the reference's own test-suite (fteikpy tests/*.py). All
# on unit-velocity, unit-spacing grids of 16 cells per axis.
REF_SOLVE_2D = {(0.0, 0.0): 3573.41870888, (3.5, 3.5): 2462.96106736}  # nsweep=2
REF_SOLVE_3D = {(0.0, 0.0, 0.0): 76631.78464590, (3.5, 3.5, 3.5): 54091.60683054}  # nsweep=3
REF_TT_3D = [  # source (0, 0, 0), nsweep=3
    ([0.0, 0.0, 0.0], 0.0),
    ([0.5, 0.5, 0.5], 0.86602540),
    ([1.5, 1.5, 1.5], 2.60631816),
    ([-1.0, -1.0, -1.0], np.nan),
    ([15.0, 0.0, 0.0], 15.0),
    ([15.0, 15.0, 0.0], 21.21320343),
    ([0.0, 15.0, 0.0], 15.0),
    ([0.0, 0.0, 15.0], 15.0),
    ([15.0, 0.0, 15.0], 21.21320343),
    ([15.0, 15.0, 15.0], 25.98076211),
    ([0.0, 15.0, 15.0], 21.21320343),
]
REF_TT_2D = [  # source (0, 0), nsweep=2
    ([0.0, 0.0], 0.0),
    ([0.5, 0.5], 0.70710678),
    ([1.5, 1.5], 2.12132034),
    ([-1.0, -1.0], np.nan),
    ([15.0, 0.0], 15.0),
    ([15.0, 15.0], 21.21320343),
    ([0.0, 15.0], 15.0),
]
REF_RAY_3D = [  # (end point, honor_grid, sum of ray coordinates), stepsize=1
    ([0.5, 0.5, 0.5], False, 1.5),
    ([0.5, 0.5, 0.5], True, 1.5),
    ([1.5, 1.5, 1.5], False, 8.30384757),
    ([1.5, 1.5, 1.5], True, 7.5),
]
REF_RAY_2D = [
    ([0.5, 0.5], False, 1.0),
    ([0.5, 0.5], True, 1.0),
    ([1.5, 1.5], False, 4.75735931),
    ([1.5, 1.5], True, 5.0),
]
REF_CORNERS_3D = [
    [0.0, 0.0, 0.0], [15.0, 0.0, 0.0], [15.0, 15.0, 0.0], [0.0, 15.0, 0.0],
    [0.0, 0.0, 15.0], [15.0, 0.0, 15.0], [15.0, 15.0, 15.0], [0.0, 15.0, 15.0],
]
REF_GRAD_3D = (  # gz, gx, gy at REF_CORNERS_3D, source (0, 0, 0), nsweep=3
    [0.0, 1.0, 0.70710678, 0.0, 0.0, 0.70710678, 0.57735027, 0.0],
    [0.0, 0.0, 0.70710678, 1.0, 0.0, 0.0, 0.57735027, 0.70710678],
    [0.0, 0.0, 0.0, 0.0, 1.0, 0.70710678, 0.57735027, 0.70710678],
)
REF_CORNERS_2D = [[0.0, 0.0], [15.0, 0.0], [15.0, 15.0], [0.0, 15.0]]
REF_GRAD_2D = ([0.0, 1.0, 0.70710678, 0.0], [0.0, 0.0, 0.70710678, 1.0])  # source (0, 0)
REF_GRAD_2D_SRC35 = (-0.70710678, -0.70710678)  # at (0, 0), source (3.5, 3.5)
# meshio round-trip test: on-node sources in the middle of small unit grids,
# default nsweep=2; traveltime sums and honor_grid ray lengths from (0, 0[, 0]).
REF_MESHIO_2D = dict(shape=(8, 10), source=(4.0, 5.0), tt_sum=378.23469225, ray_len=9)
REF_MESHIO_3D = dict(shape=(8, 10, 12), source=(4.0, 5.0, 6.0), tt_sum=6909.90160991, ray_len=14)


# A stand-in for the meshio module (not installed here): Mesh keeps what the
# export passes and turns the (type, connectivity) list into blocks with
# .type and .data, as meshio.Mesh does.
class _CellBlock:
    def __init__(self, cell_type, data):
        self.type = cell_type
        self.data = np.asarray(data)

    def __len__(self):
        return len(self.data)


class _Mesh:
    def __init__(self, points, cells, point_data=None, cell_data=None):
        self.points = np.asarray(points)
        self.cells = [_CellBlock(t, d) for t, d in cells]
        self.point_data = dict(point_data or {})
        self.cell_data = dict(cell_data or {})


def stand_in_meshio():
    import types

    mod = types.ModuleType("meshio")
    mod.Mesh = _Mesh
    return mod
