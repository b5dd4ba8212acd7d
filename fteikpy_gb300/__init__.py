"""fteikpy_gb300: fteikpy's traveltime path (FTeik Eikonal solves, gradient
fields, interpolation and ray tracing) as hand-written CUDA for GB300 (sm_103a),
behind fteikpy's own Python API.

    from fteikpy_gb300 import Eikonal3D
    tt = Eikonal3D(velocity, gridsize=(dz, dx, dy)).solve(sources, return_gradient=True)
"""

from .__about__ import __version__
from ._build import build
from ._grid import Grid2D, Grid3D, TraveltimeGrid2D, TraveltimeGrid3D
from ._helpers import get_num_threads, set_num_threads
from ._solver import Eikonal2D, Eikonal3D, autotune, solve_batch
from ._adjoint import converged, traveltimes
from ._shard import shard_bounds, sharded_traveltimes, solve_sharded
from ._io import grid_to_meshio, ray_to_meshio

__all__ = [
    "Eikonal2D",
    "Eikonal3D",
    "Grid2D",
    "Grid3D",
    "TraveltimeGrid2D",
    "TraveltimeGrid3D",
    "autotune",
    "build",
    "converged",
    "grid_to_meshio",
    "ray_to_meshio",
    "solve_batch",
    "traveltimes",
    "get_num_threads",
    "set_num_threads",
    "shard_bounds",
    "sharded_traveltimes",
    "solve_sharded",
    "__version__",
]
