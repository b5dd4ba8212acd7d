"""meshio export (``grid_to_meshio`` / ``ray_to_meshio``, fteikpy/_io.py) on
the CPU. meshio is not installed here, so a stand-in module records what the
export hands to ``meshio.Mesh``, with meshio's own conversion of the cell
list into blocks that carry ``.type`` and ``.data``.

Three references: a per-cell construction of the structured meshes written
from fteikpy/_io.py's definitions (vertex lists through
``np.ravel_multi_index``), the reference's own meshio test
(tests/test_meshio.py: point and cell counts, traveltime sum, gradient sums,
velocity sum, ray connectivity sum) on grids solved and traced by the oracle,
and the reference's errors.
"""

import sys

import numpy as np
import pytest

import fteikpy_gb300 as fp
from fteikpy_gb300 import _io
from helpers import REF_MESHIO_2D, REF_MESHIO_3D, default_max_step, model_axes, stand_in_meshio
from oracle import oracle as O


@pytest.fixture
def meshio(monkeypatch):
    mod = stand_in_meshio()
    monkeypatch.setitem(sys.modules, "meshio", mod)
    return mod


def _per_cell_2d(nx, nz, dx, dz, x0, z0):
    shape = (nx + 1, nz + 1)
    pts, cells = [], []
    for j in range(nz + 1):
        for i in range(nx + 1):
            pts.append([i * dx + x0, j * dz + z0])
    for j in range(nz):
        for i in range(nx):
            verts = [[i, j], [i + 1, j], [i + 1, j + 1], [i, j + 1]]
            cells.append([np.ravel_multi_index(v, shape, order="F") for v in verts])
    return np.array(pts), np.array(cells)


def _per_cell_3d(nx, ny, nz, dx, dy, dz, x0, y0, z0):
    shape = (nx + 1, ny + 1, nz + 1)
    pts, cells = [], []
    for i in range(nx + 1):
        for j in range(ny + 1):
            for k in range(nz + 1):
                pts.append([i * dx + x0, j * dy + y0, k * dz + z0])
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                verts = [[i, j, k], [i + 1, j, k], [i + 1, j + 1, k], [i, j + 1, k],
                         [i, j, k + 1], [i + 1, j, k + 1], [i + 1, j + 1, k + 1], [i, j + 1, k + 1]]
                cells.append([np.ravel_multi_index(v, shape) for v in verts])
    return np.array(pts), np.array(cells)


def test_structured_meshes_match_the_per_cell_construction():
    pts, cells = _io._structured_mesh_2d((3, 4), (2.0, 0.5), (1.0, -3.0))
    ref_pts, ref_cells = _per_cell_2d(4, 3, 0.5, 2.0, -3.0, 1.0)
    assert np.array_equal(pts, ref_pts)
    assert cells[0][0] == "quad" and np.array_equal(cells[0][1], ref_cells)
    pts, cells = _io._structured_mesh_3d((2, 3, 4), (2.0, 0.5, 1.5), (1.0, -3.0, 0.25))
    ref_pts, ref_cells = _per_cell_3d(3, 4, 2, 0.5, 1.5, 2.0, -3.0, 0.25, 1.0)
    assert np.array_equal(pts, ref_pts)
    assert cells[0][0] == "hexahedron" and np.array_equal(cells[0][1], ref_cells)


def _oracle_case(case):
    """The reference test's problem, solved and traced by the oracle: the
    velocity model, its traveltime grid (with gradients) and one ray."""
    nd = len(case["shape"])
    d = (1.0,) * nd
    v = np.ones(case["shape"])
    src = np.array(case["source"])
    solve = O.solve3d if nd == 3 else O.solve2d
    tt, tg, vz = solve(1.0 / v, d, src[None], 2, True)
    cls = fp.TraveltimeGrid3D if nd == 3 else fp.TraveltimeGrid2D
    grid = cls(tt[0], d, np.zeros(nd), src, tg[0], float(vz[0]))
    ax = model_axes(tt[0].shape, d, np.zeros(nd))
    ms = default_max_step(tt[0].shape, d, 1.0)
    ray = O.raytrace(ax, tg[0], np.zeros((1, nd)), src, 1.0, ms, True)[0]
    eik = (fp.Eikonal3D if nd == 3 else fp.Eikonal2D)(v, d)
    return eik, grid, ray


@pytest.mark.parametrize("case,ray_sum", [(REF_MESHIO_2D, 64.0), (REF_MESHIO_3D, 169.0)])
def test_reference_meshio_known_answers(meshio, case, ray_sum):
    eik, tt, ray = _oracle_case(case)
    mesh = fp.grid_to_meshio(eik, tt)
    mesh_ray = fp.ray_to_meshio(ray)
    shape = case["shape"]
    npts = int(np.prod(np.array(shape) + 1))
    assert len(mesh.points) == npts and mesh.points.shape[1] == 3
    assert sum(len(cell) for cell in mesh.cells) == int(np.prod(shape))
    assert mesh.point_data["Traveltime"][npts // 2] == 0.0
    assert np.allclose(mesh.point_data["Traveltime"].sum(), case["tt_sum"])
    for grad in mesh.point_data["Gradient"].T:
        assert grad[npts // 2] == 0.0
        assert np.allclose(grad.sum(), 0.0)
    assert mesh.cell_data["Velocity"][0].sum() == int(np.prod(shape))
    assert len(mesh_ray.points) == len(ray) == case["ray_len"]
    assert len(mesh_ray.cells[0].data) == len(ray) - 1
    assert mesh_ray.cells[0].data.sum() == ray_sum


def test_axes_data_names_and_several_rays(meshio):
    eik, tt, ray = _oracle_case(REF_MESHIO_3D)
    mesh = fp.grid_to_meshio(tt, eik, tt, eik)
    # the first argument sets the mesh: a traveltime grid holds nodes
    assert len(mesh.points) == np.prod(np.array(REF_MESHIO_3D["shape"]) + 1)
    assert sorted(mesh.point_data) == ["Gradient", "Gradient 2", "Traveltime", "Traveltime 2"]
    assert sorted(mesh.cell_data) == ["Velocity", "Velocity 2"]
    # (z, x, y) -> (x, y, -z); gradients likewise
    nz, nx, ny = tt.shape
    p = mesh.points.reshape(nx, ny, nz, 3)
    assert np.array_equal(p[:, 0, 0, 0], tt.xaxis) and np.array_equal(p[0, :, 0, 1], tt.yaxis)
    assert np.array_equal(p[0, 0, :, 2], -tt.zaxis)
    g = mesh.point_data["Gradient"].reshape(nx, ny, nz, 3)
    gz, gx, gy = (np.asarray(c.grid) for c in tt.gradient)
    assert np.array_equal(g[..., 0], np.transpose(gx, (1, 2, 0)))
    assert np.array_equal(g[..., 2], -np.transpose(gz, (1, 2, 0)))
    # two rays: one line block each, the second numbered after the first
    r2 = ray[:5] + 0.5
    mr = fp.ray_to_meshio(ray, r2)
    assert [c.type for c in mr.cells] == ["line", "line"]
    assert mr.cells[1].data[0, 0] == len(ray)
    assert np.array_equal(mr.points[len(ray):], np.column_stack((r2[:, 1], r2[:, 2], -r2[:, 0])))
    # 2D rays get y = 0
    m2 = fp.ray_to_meshio(np.array([[1.0, 2.0], [3.0, 4.0]]))
    assert np.array_equal(m2.points, [[2.0, 0.0, -1.0], [4.0, 0.0, -3.0]])


def test_errors_match_reference(meshio):
    with pytest.raises(ValueError, match="argument 1 is not a supported grid"):
        fp.grid_to_meshio(np.ones((3, 3)))
    eik = fp.Eikonal2D(np.ones((3, 3)), (1.0, 1.0))
    with pytest.raises(ValueError, match="argument 2 is not a supported grid"):
        fp.grid_to_meshio(eik, "grid")
    with pytest.raises(ValueError, match="argument 1 does not seem to be a ray"):
        fp.ray_to_meshio(np.ones(3))


def test_meshio_is_imported_only_when_called(monkeypatch):
    monkeypatch.setitem(sys.modules, "meshio", None)
    with pytest.raises(ImportError):
        fp.ray_to_meshio(np.ones((2, 3)))
