"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference's own outputs.

Tolerances: the kernels reproduce the reference's IEEE operation sequence
without contraction, so traveltimes, gradients, interpolated values and ray
coordinates are compared bit for bit against the C oracle, which follows the
same semantics. Against the golden fixtures produced by the pure-Python
reference (which evaluates ``x ** 0.5`` / ``x ** 2.0`` through ``pow``) the
bound is the contract's 1e-12 relative.
"""

import numpy as np
import pytest
import torch

import fteikpy_gb300 as fp
from fteikpy_gb300 import _device, _solver
from helpers import (
    REF_CORNERS_2D,
    REF_CORNERS_3D,
    REF_GRAD_2D,
    REF_GRAD_2D_SRC35,
    REF_GRAD_3D,
    REF_MESHIO_2D,
    REF_MESHIO_3D,
    REF_RAY_2D,
    REF_RAY_3D,
    REF_SOLVE_2D,
    REF_SOLVE_3D,
    REF_TT_2D,
    REF_TT_3D,
    default_max_step,
    max_rel,
    model_axes,
    stand_in_meshio,
)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the contract: max relative error against the reference


def layered3d(shape, seed, d=(10.0, 10.0, 10.0)):
    rng = np.random.default_rng(seed)
    nz = shape[0]
    tops = np.sort(rng.integers(1, nz, 3))
    vels = np.sort(rng.uniform(1500.0, 4500.0, 4))
    v = vels[np.searchsorted(tops, np.arange(nz), side="right")][:, None, None] * np.ones(shape)
    v *= 1.0 + 0.05 * rng.uniform(-1.0, 1.0, shape)
    return v


def rand_sources(rng, shape, d, n, origin):
    ext = np.array(shape) * np.array(d)
    return origin + rng.uniform(0.0, 1.0, (n, len(shape))) * ext


def bitwise(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


# ---------------------------------------------------------------- known answers


@pytest.mark.parametrize("src", list(REF_SOLVE_3D))
def test_known_answer_solve3d(src):
    eik = fp.Eikonal3D(np.ones((16, 16, 16)), (1.0, 1.0, 1.0))
    tt = eik.solve(list(src), nsweep=3)
    assert np.allclose(tt.grid.sum(), REF_SOLVE_3D[src], atol=1e-8)
    tts = eik.solve([list(s) for s in REF_SOLVE_3D], nsweep=3)
    assert np.allclose([t.grid.sum() for t in tts], list(REF_SOLVE_3D.values()), atol=1e-8)


@pytest.mark.parametrize("src", list(REF_SOLVE_2D))
def test_known_answer_solve2d(src):
    eik = fp.Eikonal2D(np.ones((16, 16)), (1.0, 1.0))
    tt = eik.solve(list(src), nsweep=2)
    assert np.allclose(tt.grid.sum(), REF_SOLVE_2D[src], atol=1e-8)
    tts = eik.solve([list(s) for s in REF_SOLVE_2D], nsweep=2)
    assert np.allclose([t.grid.sum() for t in tts], list(REF_SOLVE_2D.values()), atol=1e-8)


def test_known_answer_call_gradient_raytrace_3d():
    eik = fp.Eikonal3D(np.ones((16, 16, 16)), (1.0, 1.0, 1.0))
    assert eik([0.0, 0.0, 0.0]) == 1.0
    assert np.isnan(eik([-1.0, -1.0, -1.0]))
    assert np.allclose(eik(REF_CORNERS_3D), np.ones(8))
    tt = eik.solve([0.0, 0.0, 0.0], nsweep=3, return_gradient=True)
    for p, ref in REF_TT_3D:
        got = tt(p)
        assert (np.isnan(got) and np.isnan(ref)) or np.allclose(got, ref, atol=1e-8)
    for c in range(3):
        assert np.allclose(tt.gradient[c](REF_CORNERS_3D), REF_GRAD_3D[c], atol=1e-8)
        assert np.isnan(tt.gradient[c]([-1.0, -1.0, -1.0]))
    for end, hg, s in REF_RAY_3D:
        assert np.allclose(tt.raytrace(end, stepsize=1.0, honor_grid=hg).sum(), s, atol=1e-8)
    for hg in (False, True):
        ends = [e for e, h, _ in REF_RAY_3D if h == hg]
        sums = [s for _, h, s in REF_RAY_3D if h == hg]
        rays = tt.raytrace(ends, stepsize=1.0, honor_grid=hg)
        assert np.allclose([r.sum() for r in rays], sums, atol=1e-8)


def test_known_answer_call_gradient_raytrace_2d():
    eik = fp.Eikonal2D(np.ones((16, 16)), (1.0, 1.0))
    assert eik([0.0, 0.0]) == 1.0
    assert np.allclose(eik(REF_CORNERS_2D), np.ones(4))
    tt = eik.solve([0.0, 0.0], nsweep=2, return_gradient=True)
    for p, ref in REF_TT_2D:
        got = tt(p)
        assert (np.isnan(got) and np.isnan(ref)) or np.allclose(got, ref, atol=1e-8)
    for c in range(2):
        assert np.allclose(tt.gradient[c](REF_CORNERS_2D), REF_GRAD_2D[c], atol=1e-8)
    for end, hg, s in REF_RAY_2D:
        assert np.allclose(tt.raytrace(end, stepsize=1.0, honor_grid=hg).sum(), s, atol=1e-8)
    tt = eik.solve([3.5, 3.5], nsweep=2, return_gradient=True)
    assert np.allclose([tt.gradient[c]([0.0, 0.0]) for c in range(2)], REF_GRAD_2D_SRC35, atol=1e-8)


@pytest.mark.parametrize("case,ray_sum", [(REF_MESHIO_2D, 64.0), (REF_MESHIO_3D, 169.0)])
def test_known_answer_meshio(case, ray_sum, monkeypatch):
    """The reference's meshio test (tests/test_meshio.py) on this library's
    solve and rays, through grid_to_meshio / ray_to_meshio with a stand-in
    for the meshio module."""
    import sys

    monkeypatch.setitem(sys.modules, "meshio", stand_in_meshio())
    nd = len(case["shape"])
    cls = fp.Eikonal3D if nd == 3 else fp.Eikonal2D
    eik = cls(np.ones(case["shape"]), (1.0,) * nd)
    tt = eik.solve(case["source"], return_gradient=True)
    assert np.allclose(tt.grid.sum(), case["tt_sum"], atol=1e-8)
    ray = tt.raytrace(np.zeros(nd), honor_grid=True)
    assert len(ray) == case["ray_len"]
    mesh, mesh_ray = fp.grid_to_meshio(eik, tt), fp.ray_to_meshio(ray)
    npts = int(np.prod(np.array(case["shape"]) + 1))
    assert len(mesh.points) == npts
    assert sum(len(cell) for cell in mesh.cells) == int(np.prod(case["shape"]))
    assert mesh.point_data["Traveltime"][npts // 2] == 0.0
    assert np.allclose(mesh.point_data["Traveltime"].sum(), case["tt_sum"])
    for grad in mesh.point_data["Gradient"].T:
        assert grad[npts // 2] == 0.0
        assert np.allclose(grad.sum(), 0.0)
    assert mesh.cell_data["Velocity"][0].sum() == int(np.prod(case["shape"]))
    assert len(mesh_ray.points) == len(ray)
    assert len(mesh_ray.cells[0].data) == len(ray) - 1
    assert mesh_ray.cells[0].data.sum() == ray_sum


# ------------------------------------------------------------- golden fixtures


@pytest.mark.parametrize("nd", [2, 3])
def test_golden_solve_and_interp(nd, golden2d, golden3d):
    g = golden3d if nd == 3 else golden2d
    cls = fp.Eikonal3D if nd == 3 else fp.Eikonal2D
    eik = cls(g["velocity"], g["gridsize"], g["origin"])
    tts = eik.solve(g["sources"], nsweep=int(g["nsweep"]), return_gradient=True)
    tt = np.stack([t.grid for t in tts])
    assert max_rel(tt, g["tt"]) <= TOL
    grad = np.stack([t._gradient.cpu().numpy() for t in tts])
    assert np.abs(grad - g["ttgrad"]).max() <= 1e-10
    assert np.array_equal([t._vzero for t in tts], g["vzero"])
    for s, t in enumerate(tts):
        assert max_rel(t(g["points"]), g["vinterp"][s]) <= TOL
        for c in range(nd):
            gi = t.gradient[c](g["points"])
            assert np.array_equal(np.isnan(gi), np.isnan(g["gradinterp"][s][c]))
            assert np.nanmax(np.abs(gi - g["gradinterp"][s][c])) <= 1e-10
        for hg in (0, 1):
            rays = t.raytrace(g["receivers"], honor_grid=bool(hg))
            assert np.array_equal([len(r) for r in rays], g[f"raylen_s{s}_hg{hg}"])
            assert np.abs(np.concatenate(rays) - g[f"rays_s{s}_hg{hg}"]).max() <= 1e-9
    assert max_rel(eik(g["points"]), g["velinterp"]) == 0.0
    if nd == 3:
        t1 = eik.solve(g["sources"][0], nsweep=1, return_gradient=True)
        assert max_rel(t1.grid, g["tt_nsweep1"]) <= TOL
        rays = tts[0].raytrace(g["receivers"], stepsize=4.0)
        assert np.array_equal([len(r) for r in rays], g["raylen_s0_step4"])
    else:
        t3 = eik.solve(g["sources"][:2], nsweep=3, return_gradient=True)
        assert max_rel(np.stack([t.grid for t in t3]), g["tt_nsweep3"]) <= TOL
        rays = tts[0].raytrace(g["receivers"], stepsize=3.0)
        assert np.array_equal([len(r) for r in rays], g["raylen_s0_step3"])


# ------------------------------------------------- bitwise against the oracle


@pytest.mark.parametrize(
    "shape,d,nsrc,nsweep,seed",
    [
        ((12, 14, 16), (9.0, 11.0, 10.0), 3, 2, 0),
        ((2, 2, 2), (1.0, 1.0, 1.0), 2, 2, 1),
        ((3, 17, 5), (4.0, 1.5, 2.5), 4, 3, 2),
        ((40, 33, 47), (10.0, 10.0, 10.0), 5, 2, 3),
        ((25, 9, 70), (7.0, 13.0, 5.0), 2, 1, 4),
        ((30, 40, 24), (10.0, 10.0, 10.0), 1, 0, 5),
        # micrometre spacing: slowness x spacing < 1e-9 disables the Big skip
        ((10, 12, 9), (1e-6, 2e-6, 1.5e-6), 2, 2, 6),
        ((64, 20, 33), (5.0, 5.0, 5.0), 3, 2, 7),
    ],
)
def test_solve3d_bitwise_vs_oracle(shape, d, nsrc, nsweep, seed):
    rng = np.random.default_rng(seed)
    v = layered3d(shape, seed)
    src = rand_sources(rng, shape, d, nsrc, np.zeros(3))
    src[0, 0] = 0.0  # a surface source
    if nsrc > 1:
        src[1] = np.floor(src[1] / d) * d  # on a node
    tt_o, tg_o, vz_o = O.solve3d(1.0 / v, d, src, nsweep, True)
    eik = fp.Eikonal3D(v, d)
    tts = eik.solve(src, nsweep=nsweep, return_gradient=True)
    tt = np.stack([t.grid for t in tts])
    tg = np.stack([t._gradient.cpu().numpy() for t in tts])
    assert max_rel(tt, tt_o) <= TOL
    assert bitwise(tt, tt_o), f"{(tt != tt_o).sum()} of {tt.size} traveltimes differ in bits"
    assert bitwise(tg, tg_o), f"{(tg != tg_o).sum()} gradient components differ in bits"
    assert np.array_equal([t._vzero for t in tts], vz_o)
    # without gradients the traveltimes are the same
    tt_ng = np.stack([t.grid for t in eik.solve(src, nsweep=nsweep)])
    assert bitwise(tt_ng, tt_o)


@pytest.mark.parametrize("nsrc", [1, 7, 64])
def test_solve3d_batched_equals_single(nsrc):
    rng = np.random.default_rng(100 + nsrc)
    shape, d = (20, 26, 30), (10.0, 10.0, 10.0)
    v = layered3d(shape, 7)
    src = rand_sources(rng, shape, d, nsrc, np.zeros(3))
    eik = fp.Eikonal3D(v, d)
    batch = eik.solve(src, nsweep=2, return_gradient=True)
    for i in sorted({0, nsrc // 2, nsrc - 1}):
        one = eik.solve(src[i], nsweep=2, return_gradient=True)
        assert bitwise(one.grid, batch[i].grid)
        assert bitwise(one._gradient.cpu().numpy(), batch[i]._gradient.cpu().numpy())
    tt_o, _, _ = O.solve3d(1.0 / v, d, src[[0, nsrc - 1]], 2, False)
    assert bitwise(batch[0].grid, tt_o[0]) and bitwise(batch[-1].grid, tt_o[1])


# 2D kernels: (sweep2d_warp, sweep2d_speculate) -- a block per source with
# speculated updates (the default up to one source per SM), the same without
# them, one warp per source with and without them, one thread per source
KERNELS_2D = {"team": (2, -1), "team_nospec": (2, 0), "warp": (1, -1), "warp_nospec": (1, 0),
              "thread": (0, -1)}


def _set_2d(lib, keys, kernel):
    warp, spec = KERNELS_2D[kernel]
    assert lib.fteik_set_option(b"sweep2d_keys", keys) == 0
    assert lib.fteik_set_option(b"sweep2d_warp", warp) == 0
    assert lib.fteik_set_option(b"sweep2d_speculate", spec) == 0


def _reset_2d(lib):
    for name in (b"sweep2d_keys", b"sweep2d_warp", b"sweep2d_speculate"):
        lib.fteik_set_option(name, -1)


@pytest.mark.parametrize(
    "shape,d,nsrc,nsweep,seed",
    [
        ((24, 32), (10.0, 8.0), 5, 2, 0),
        ((2, 2), (1.0, 1.0), 2, 2, 1),
        ((60, 45), (5.0, 7.0), 9, 3, 2),
        ((13, 90), (10.0, 10.0), 3, 1, 3),
    ],
)
@pytest.mark.parametrize("keys", [-1, 0])
@pytest.mark.parametrize("kernel", list(KERNELS_2D))
def test_solve2d_bitwise_vs_oracle(shape, d, nsrc, nsweep, seed, keys, kernel):
    """Every 2D kernel (a block per source whose producer warps precompute the
    rows' tv-independent terms ahead of the chain, and one warp per source that
    precomputes them between stretches of it, each with and without the
    speculated updates; one thread per source) and both comparison paths
    (integer keys, the default for sources whose first propagation is finite;
    IEEE comparisons) against the oracle, bit for bit."""
    from fteikpy_gb300 import _lib

    lib = _lib.load()
    _set_2d(lib, keys, kernel)
    try:
        _solve2d_bitwise_case(shape, d, nsrc, nsweep, seed)
    finally:
        _reset_2d(lib)


def _solve2d_bitwise_case(shape, d, nsrc, nsweep, seed):
    rng = np.random.default_rng(seed)
    v = 1500.0 + 30.0 * np.arange(shape[0])[:, None] * np.ones(shape)
    v *= 1.0 + 0.1 * rng.uniform(-1.0, 1.0, shape)
    src = rand_sources(rng, shape, d, nsrc, np.zeros(2))
    src[0, 0] = 0.0
    if nsrc > 1:
        src[1] = np.floor(src[1] / d) * d
    tt_o, tg_o, vz_o = O.solve2d(1.0 / v, d, src, nsweep, True)
    tts = fp.Eikonal2D(v, d).solve(src, nsweep=nsweep, return_gradient=True)
    tt = np.stack([t.grid for t in tts])
    tg = np.stack([t._gradient.cpu().numpy() for t in tts])
    assert max_rel(tt, tt_o) <= TOL
    assert bitwise(tt, tt_o), f"{(tt != tt_o).sum()} of {tt.size} traveltimes differ in bits"
    assert bitwise(tg, tg_o)


def test_interp_and_rays_bitwise_vs_oracle():
    rng = np.random.default_rng(9)
    shape, d, og = (20, 24, 28), (10.0, 12.0, 8.0), np.array([3.0, -5.0, 7.0])
    v = layered3d(shape, 9)
    src = og + np.array([0.0, 131.7, 97.3])
    eik = fp.Eikonal3D(v, d, og)
    tt = eik.solve(src, nsweep=2, return_gradient=True)
    tg = tt._gradient.cpu().numpy()
    ax = model_axes(tt.shape, d, og)
    hi = og + np.array(d) * (np.array(tt.shape) - 1)
    pts = rng.uniform(og - 3.0, hi + 3.0, (2000, 3))
    assert bitwise(tt(pts), O.vinterp(ax, tt.grid, pts, src, tt._vzero))
    for c in range(3):
        assert bitwise(tt.gradient[c](pts), O.interp(ax, tg[..., c], pts, stride=3))
    rec = np.column_stack([np.full(300, og[0]), rng.uniform(og[1], hi[1], 300), rng.uniform(og[2], hi[2], 300)])
    for hg in (False, True):
        stepsize = min(d)
        ms = default_max_step(tt.shape, d, stepsize)
        # Some honor_grid rays walk along cell faces until max_step in the
        # reference as well: both sides must fail on exactly those rays.
        fails = []
        for i in range(len(rec)):
            try:
                O.raytrace(ax, tg, rec[i : i + 1], src, stepsize, ms, hg)
            except RuntimeError:
                fails.append(i)
        for i in fails:
            with pytest.raises(RuntimeError, match="maximum number of steps reached"):
                tt.raytrace(rec[i], honor_grid=hg)
        keep = np.setdiff1d(np.arange(len(rec)), fails)
        got = tt.raytrace(rec[keep], honor_grid=hg)
        ref = O.raytrace(ax, tg, rec[keep], src, stepsize, ms, hg)
        assert [len(r) for r in got] == [len(r) for r in ref]
        assert bitwise(np.concatenate(got), np.concatenate(ref))


def test_errors_match_reference():
    eik = fp.Eikonal3D(np.ones((6, 6, 6)), (1.0, 1.0, 1.0))
    with pytest.raises(ValueError, match="source out of bound"):
        eik.solve([7.0, 0.0, 0.0])
    tt = eik.solve([0.0, 0.0, 0.0], return_gradient=True)
    with pytest.raises(ValueError, match="end point out of bound"):
        tt.raytrace([[1.0, 1.0, 1.0], [7.0, 0.0, 0.0]])
    with pytest.raises(RuntimeError, match="maximum number of steps reached"):
        tt.raytrace([6.0, 6.0, 6.0], stepsize=0.1, max_step=5)
    with pytest.raises(ValueError, match="no gradient grid"):
        eik.solve([0.0, 0.0, 0.0]).gradient


def test_device_wait_timeout_is_reported_and_recoverable():
    """A dependency wait that runs out reports an error status, the kernel
    returns, and the context stays usable (no GPU fault, no hang)."""
    v = layered3d((30, 40, 48), 11)
    slow = _device.slowness(_device.to_device(v))
    src = np.array([[0.0, 150.0, 200.0]])
    with pytest.raises(RuntimeError, match="timed out"):
        _solver.solve3d_device(slow, (10.0, 10.0, 10.0), src, 2, True, spin_limit=1)
    tt, _, _ = _solver.solve3d_device(slow, (10.0, 10.0, 10.0), src, 2, True)
    tt_o, _, _ = O.solve3d(1.0 / v, (10.0, 10.0, 10.0), src, 2, False)
    assert bitwise(tt.cpu().numpy(), tt_o)


def test_torch_cuda_grid_is_used_in_place():
    v = layered3d((10, 12, 14), 12)
    vt = torch.as_tensor(v, device="cuda")
    a = fp.Eikonal3D(vt, (10.0, 10.0, 10.0)).solve([0.0, 30.0, 40.0])
    b = fp.Eikonal3D(v, (10.0, 10.0, 10.0)).solve([0.0, 30.0, 40.0])
    assert bitwise(a.grid, b.grid)


@pytest.mark.parametrize("coef", [0, 1])
def test_solve3d_both_coefficient_sources(coef):
    """The sweep's slowness factors read from precomputed arrays or derived
    from the slowness cells give the same bits."""
    from fteikpy_gb300 import _lib

    lib = _lib.load()
    assert lib.fteik_set_option(b"sweep_coef", coef) == 0
    try:
        rng = np.random.default_rng(21)
        shape, d = (20, 26, 30), (9.0, 10.0, 11.0)
        v = layered3d(shape, 21)
        src = rand_sources(rng, shape, d, 3, np.zeros(3))
        tt_o, tg_o, _ = O.solve3d(1.0 / v, d, src, 2, True)
        tts = fp.Eikonal3D(v, d).solve(src, nsweep=2, return_gradient=True)
        assert bitwise(np.stack([t.grid for t in tts]), tt_o)
        assert bitwise(np.stack([t._gradient.cpu().numpy() for t in tts]), tg_o)
    finally:
        lib.fteik_set_option(b"sweep_coef", -1)


def test_rays_with_one_four_and_32_lanes_per_ray_agree():
    """Large ray batches run one lane per ray, smaller ones four (one axis per
    lane), one source's receivers a warp per ray: the same rays bit for bit,
    and the oracle's."""
    from fteikpy_gb300 import _lib
    from fteikpy_gb300._grid import trace_rays

    rng = np.random.default_rng(31)
    shape, d = (20, 30, 25), (10.0, 10.0, 10.0)
    v = layered3d(shape, 31)
    src = np.array([0.0, 140.0, 120.0])
    tt = fp.Eikonal3D(v, d).solve(src, nsweep=2, return_gradient=True)
    ax = [_device.to_device(a) for a in O.axes(tt.shape, d, np.zeros(3))]
    ext = np.array(shape) * np.array(d)
    ends = rng.uniform(0.0, 1.0, (16400, 3)) * ext
    g = tt._gradient.contiguous()
    max_dist = 2.0 * sum((n * h) ** 2 for n, h in zip(tt.shape, d)) ** 0.5
    max_step = int(max_dist / 10.0)
    many = trace_rays(3, ax, g, None, ends, src[None], 10.0, max_step, False)
    lib = _lib.load()
    try:
        for lanes in (-1, 4, 32):
            assert lib.fteik_set_option(b"ray_lanes", lanes) == 0
            few = trace_rays(3, ax, g, None, ends[:400], src[None], 10.0, max_step, False)
            assert all(np.array_equal(a, b) for a, b in zip(many[:400], few)), lanes
    finally:
        lib.fteik_set_option(b"ray_lanes", -1)
    tg_o = O.solve3d(1.0 / v, d, [src], 2, True)[1][0]
    sample = rng.choice(len(ends), 40, replace=False)
    ref = O.raytrace(O.axes(tt.shape, d, np.zeros(3)), tg_o, ends[sample], src, 10.0, max_step,
                     False)
    assert all(np.array_equal(many[i], r) for i, r in zip(sample, ref))


@pytest.mark.parametrize(
    "nd,d,og,stepsize",
    [
        # spacings that are not exact in binary: x2 - x1 differs from cell to
        # cell in the last bits, so the blends divide by each cell's volume
        (3, (0.3, 0.7, 0.5), (0.3, -1.1, 0.7), None),
        (3, (0.7, 0.3, 0.9), (0.1, 0.3, -0.7), None),
        # one exact spacing per axis (the constant-volume division), a step
        # that is not a multiple of the spacing
        (3, (10.0, 12.0, 8.0), (3.0, -5.0, 7.0), 3.3),
        (2, (0.3, 0.7), (0.3, 0.7), None),
        (2, (5.0, 7.0), (-1.0, 2.0), None),
    ],
)
@pytest.mark.parametrize("lanes", [-1, 4, 1])
def test_rays_bitwise_vs_oracle_on_exact_and_inexact_axes(nd, d, og, stepsize, lanes):
    """Rays (no honor_grid) against the oracle bit for bit, on axes where every
    cell has the same volume and on axes where the volumes differ by
    rounding, with each ray kernel (by default 120 rays run a warp per ray)."""
    from fteikpy_gb300 import _lib

    lib = _lib.load()
    assert lib.fteik_set_option(b"ray_lanes", lanes) == 0
    try:
        _rays_bitwise_case(nd, d, og, stepsize)
    finally:
        lib.fteik_set_option(b"ray_lanes", -1)


def _rays_bitwise_case(nd, d, og, stepsize):
    rng = np.random.default_rng(17)
    shape = (14, 17, 19)[:nd]
    og = np.array(og)
    v = 1500.0 + 40.0 * np.arange(shape[0]).reshape((-1,) + (1,) * (nd - 1)) * np.ones(shape)
    v *= 1.0 + 0.05 * rng.uniform(-1.0, 1.0, shape)
    ext = np.array(d) * np.array(shape)
    src = og + np.concatenate([[0.0], rng.uniform(0.2, 0.8, nd - 1) * ext[1:]])
    cls = fp.Eikonal3D if nd == 3 else fp.Eikonal2D
    tt = cls(v, d, og).solve(src, nsweep=2, return_gradient=True)
    tg = tt._gradient.cpu().numpy()
    ax = model_axes(tt.shape, d, og)
    hi = og + np.array(d) * (np.array(tt.shape) - 1)
    rec = np.column_stack(
        [np.full(120, og[0])] + [rng.uniform(og[q], hi[q], 120) for q in range(1, nd)]
    )
    rec[:5, 0] = hi[0]  # the far edge of the first axis: the last-node extension
    step = min(d) if stepsize is None else stepsize
    ms = default_max_step(tt.shape, d, step)
    # rays the reference cannot finish (max_step) must fail here as well
    fails = []
    for i in range(len(rec)):
        try:
            O.raytrace(ax, tg, rec[i : i + 1], src, step, ms, False)
        except RuntimeError:
            fails.append(i)
    for i in fails:
        with pytest.raises(RuntimeError, match="maximum number of steps reached"):
            tt.raytrace(rec[i], stepsize=step)
    keep = np.setdiff1d(np.arange(len(rec)), fails)
    got = tt.raytrace(rec[keep], stepsize=step)
    ref = O.raytrace(ax, tg, rec[keep], src, step, ms, False)
    assert [len(r) for r in got] == [len(r) for r in ref]
    assert bitwise(np.concatenate(got), np.concatenate(ref))


@pytest.mark.parametrize("keys", [-1, 0])
@pytest.mark.parametrize("kernel", list(KERNELS_2D))
def test_solve2d_sources_on_the_far_boundaries(keys, kernel):
    """Sources on the bottom and right model edges (where the reference's first
    propagation divides by zero, _fteik2d.py:444-445) next to interior ones,
    in one launch: both comparison paths against the oracle, bit for bit."""
    from fteikpy_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(3)
    shape, d = (40, 36), (10.0, 8.0)
    v = 1500.0 + 30.0 * np.arange(shape[0])[:, None] * np.ones(shape)
    v *= 1.0 + 0.1 * rng.uniform(-1.0, 1.0, shape)
    zmax, xmax = shape[0] * d[0], shape[1] * d[1]
    src = np.array([[zmax, 123.3], [55.5, 100.1], [zmax, xmax], [0.0, 77.7], [133.0, xmax],
                    [zmax, 0.0], [211.1, 150.0]])
    _set_2d(lib, keys, kernel)
    try:
        tts = fp.Eikonal2D(v, d).solve(src, nsweep=2, return_gradient=True)
    finally:
        _reset_2d(lib)
    tt_o, tg_o, vz_o = O.solve2d(1.0 / v, d, src, 2, True)
    assert bitwise(np.stack([t.grid for t in tts]), tt_o)
    assert bitwise(np.stack([t._gradient.cpu().numpy() for t in tts]), tg_o)


def test_solve2d_block_kernel_wait_gives_up_then_recovers():
    """The waits between the warps of the block-per-source 2D kernel are
    bounded. With the bound at 0 ns the chain's first wait for a precomputed
    chunk gives up, the block stops, and the solve reports the device-side
    timeout (the reference-facing RuntimeError). The next solve, with the
    default bound, equals the oracle bit for bit."""
    from fteikpy_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(5)
    shape, d = (70, 50), (10.0, 10.0)
    v = 1500.0 + 20.0 * np.arange(shape[0])[:, None] * np.ones(shape)
    v *= 1.0 + 0.05 * rng.uniform(-1.0, 1.0, shape)
    src = np.array([[35.5, 260.2], [401.0, 77.3]])
    assert lib.fteik_set_option(b"sweep2d_warp", 2) == 0
    try:
        assert lib.fteik_set_option(b"sweep2d_wait_ns", 0) == 0
        with pytest.raises(RuntimeError, match="timed out"):
            fp.Eikonal2D(v, d).solve(src, nsweep=2)
        assert lib.fteik_set_option(b"sweep2d_wait_ns", -1) == 0
        tts = fp.Eikonal2D(v, d).solve(src, nsweep=2, return_gradient=True)
    finally:
        lib.fteik_set_option(b"sweep2d_wait_ns", -1)
        lib.fteik_set_option(b"sweep2d_warp", -1)
    tt_o, tg_o, _ = O.solve2d(1.0 / v, d, src, 2, True)
    assert bitwise(np.stack([t.grid for t in tts]), tt_o)
    assert bitwise(np.stack([t._gradient.cpu().numpy() for t in tts]), tg_o)
