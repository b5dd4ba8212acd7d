"""meshio export of grids and rays, mirroring fteikpy/_io.py (the step after the
solve: writing velocity models, traveltime and gradient grids and ray paths
for visualisation).

Same functions, argument meaning, errors and mesh layout as the reference:
structured quad (2D) or hexahedron (3D) meshes whose points are the grid
nodes, x fastest in 2D and z fastest in 3D; velocities as cell data,
traveltimes and gradients as point data; axes swapped from (z, x[, y]) to
(x, y, z) with z turned into elevation. meshio is imported when called, as in
the reference, so the rest of the package works without it. The mesh
connectivity is built with array arithmetic instead of per-cell lists; the
resulting arrays are the reference's.
"""

import numpy as np

from ._grid import TraveltimeGrid2D, TraveltimeGrid3D
from ._solver import Eikonal2D, Eikonal3D

_GRIDS = (Eikonal2D, Eikonal3D, TraveltimeGrid2D, TraveltimeGrid3D)


def grid_to_meshio(*args):
    """Return a ``meshio.Mesh`` of the given grids (fteikpy/_io.py:7-105).

    Each argument is an ``Eikonal2D``/``Eikonal3D`` (its velocity model
    becomes cell data "Velocity", "Velocity 2", ...) or a
    ``TraveltimeGrid2D``/``TraveltimeGrid3D`` (point data "Traveltime", and
    "Gradient" when it holds gradients). The first argument sets the mesh.
    """
    import meshio

    for i, arg in enumerate(args):
        if not isinstance(arg, _GRIDS):
            raise ValueError(f"argument {i + 1} is not a supported grid")
    first = args[0]
    ndim = len(first.shape)
    node_grid = isinstance(first, (TraveltimeGrid2D, TraveltimeGrid3D))
    # cells per axis: a traveltime grid holds nodes, a velocity model cells
    ncell = [n - 1 if node_grid else n for n in first.shape]
    if ndim == 2:
        points, cells = _structured_mesh_2d(ncell, first.gridsize, first.origin)
        points = np.column_stack((points, np.zeros(len(points))))[:, [0, 2, 1]]
    else:
        points, cells = _structured_mesh_3d(ncell, first.gridsize, first.origin)
    points[:, 2] *= -1.0  # depth -> elevation

    point_data, cell_data = {}, {}
    nvel = ntt = 0
    for arg in args:
        if isinstance(arg, (Eikonal2D, Eikonal3D)):
            nvel += 1
            cell_data["Velocity" if nvel == 1 else f"Velocity {nvel}"] = [
                _ravel_grid(arg.grid, ndim)
            ]
        else:
            ntt += 1
            suffix = "" if ntt == 1 else f" {ntt}"
            point_data["Traveltime" + suffix] = _ravel_grid(arg.grid, ndim)
            if arg._gradient is not None:
                grad = np.column_stack([_ravel_grid(g.grid, ndim) for g in arg.gradient])
                if ndim == 2:
                    grad = np.column_stack((grad, np.zeros(len(points))))
                grad = grad[:, [1, 2, 0]]
                grad[:, 2] *= -1.0
                point_data["Gradient" + suffix] = grad
    return meshio.Mesh(points, cells, point_data, cell_data)


def ray_to_meshio(*args):
    """Return a ``meshio.Mesh`` of ray paths, one "line" cell block per ray
    (fteikpy/_io.py:108-148). Each argument is a ray as ``raytrace`` returns
    it: an (npoints, ndim) array in (z, x[, y]) order."""
    import meshio

    for i, arg in enumerate(args):
        if np.ndim(arg) != 2:
            raise ValueError(f"argument {i + 1} does not seem to be a ray")
    ndim = np.shape(args[0])[1]
    rays = [np.asarray(ray) for ray in args]
    cells, start = [], 0
    for ray in rays:
        idx = np.arange(len(ray)) + start
        cells.append(("line", np.column_stack((idx[:-1], idx[1:]))))
        start += len(ray)
    points = np.concatenate(rays, axis=0)
    if ndim == 2:
        points = np.column_stack((points, np.zeros(len(points))))
    points = np.array(points)[:, [1, 2, 0]]  # (z, x, y) -> (x, y, z)
    points[:, 2] *= -1.0  # depth -> elevation
    return meshio.Mesh(points, cells)


def _structured_mesh_2d(ncell, gridsize, origin):
    """Nodes (x fastest) and quads of an nz x nx cell grid, as
    fteikpy/_io.py:_generate_mesh_2d lays them out."""
    nz, nx = ncell
    dz, dx = gridsize
    z0, x0 = origin
    x = np.arange(nx + 1) * dx + x0
    z = np.arange(nz + 1) * dz + z0
    X, Z = np.meshgrid(x, z, indexing="xy")  # [z][x]: x fastest once flattened
    points = np.column_stack((X.ravel(), Z.ravel())).astype(float)
    i, j = np.meshgrid(np.arange(nx), np.arange(nz), indexing="xy")
    base = (i + j * (nx + 1)).ravel().astype(np.int64)
    quads = np.column_stack((base, base + 1, base + nx + 2, base + nx + 1))
    return points, [("quad", quads)]


def _structured_mesh_3d(ncell, gridsize, origin):
    """Nodes (z fastest) and hexahedra of an nz x nx x ny cell grid, as
    fteikpy/_io.py:_generate_mesh_3d lays them out."""
    nz, nx, ny = ncell
    dz, dx, dy = gridsize
    z0, x0, y0 = origin
    x = np.arange(nx + 1) * dx + x0
    y = np.arange(ny + 1) * dy + y0
    z = np.arange(nz + 1) * dz + z0
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    points = np.column_stack((X.ravel(), Y.ravel(), Z.ravel())).astype(float)
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    sj, si = nz + 1, (ny + 1) * (nz + 1)  # node index = i * si + j * sj + k
    base = (I * si + J * sj + K).ravel().astype(np.int64)
    hexa = np.column_stack(
        (base, base + si, base + si + sj, base + sj,
         base + 1, base + si + 1, base + si + sj + 1, base + sj + 1)
    )
    return points, [("hexahedron", hexa)]


def _ravel_grid(grid, ndim):
    """Grid values in the mesh's point (or cell) order."""
    return grid.ravel() if ndim == 2 else np.transpose(grid, axes=[1, 2, 0]).ravel()
