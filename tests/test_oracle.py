"""Pin the CPU oracle against the reference (CPU only, no GPU).

Two anchors: the known answers of the reference's own test-suite, and the
golden fixtures produced by importing the reference itself
(tests/golden/make_golden.py).
"""

import numpy as np
import pytest

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
)
from oracle import oracle as O

# The oracle restates the reference with sqrt / x*x where the pure-Python
# reference calls pow(); the two differ in the last bit for a few inputs.
TOL_ORACLE_VS_REF = 1e-13


@pytest.mark.parametrize("src", list(REF_SOLVE_3D))
def test_known_answer_solve3d(src):
    tt, _, _ = O.solve3d(np.ones((16, 16, 16)), (1.0, 1.0, 1.0), [src], nsweep=3)
    assert np.allclose(tt[0].sum(), REF_SOLVE_3D[src], atol=1e-8)


@pytest.mark.parametrize("src", list(REF_SOLVE_2D))
def test_known_answer_solve2d(src):
    tt, _, _ = O.solve2d(np.ones((16, 16)), (1.0, 1.0), [src], nsweep=2)
    assert np.allclose(tt[0].sum(), REF_SOLVE_2D[src], atol=1e-8)


def test_known_answer_batched_matches_single():
    srcs = np.array(list(REF_SOLVE_3D))
    tt, _, _ = O.solve3d(np.ones((16, 16, 16)), (1.0, 1.0, 1.0), srcs, nsweep=3)
    assert np.allclose(tt.sum(axis=(1, 2, 3)), list(REF_SOLVE_3D.values()), atol=1e-8)


def test_known_answer_interp_and_rays_3d():
    tt, tg, vz = O.solve3d(np.ones((16, 16, 16)), (1.0, 1.0, 1.0), [[0.0, 0.0, 0.0]], 3, True)
    ax = model_axes(tt.shape[1:], (1.0,) * 3, np.zeros(3))
    pts = np.array([p for p, _ in REF_TT_3D])
    got = O.vinterp(ax, tt[0], pts, np.zeros(3), vz[0])
    ref = np.array([t for _, t in REF_TT_3D])
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.allclose(got[~np.isnan(ref)], ref[~np.isnan(ref)], atol=1e-8)
    for c in range(3):
        g = O.interp(ax, tg[0][..., c], REF_CORNERS_3D, stride=3)
        assert np.allclose(g, REF_GRAD_3D[c], atol=1e-8)
    for end, hg, s in REF_RAY_3D:
        ray = O.raytrace(ax, tg[0], [end], np.zeros(3), 1.0, default_max_step(tt.shape[1:], (1,) * 3, 1.0), hg)[0]
        assert np.allclose(ray.sum(), s, atol=1e-8)


def test_known_answer_interp_and_rays_2d():
    tt, tg, vz = O.solve2d(np.ones((16, 16)), (1.0, 1.0), [[0.0, 0.0]], 2, True)
    ax = model_axes(tt.shape[1:], (1.0,) * 2, np.zeros(2))
    pts = np.array([p for p, _ in REF_TT_2D])
    got = O.vinterp(ax, tt[0], pts, np.zeros(2), vz[0])
    ref = np.array([t for _, t in REF_TT_2D])
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.allclose(got[~np.isnan(ref)], ref[~np.isnan(ref)], atol=1e-8)
    for c in range(2):
        g = O.interp(ax, tg[0][..., c], REF_CORNERS_2D, stride=2)
        assert np.allclose(g, REF_GRAD_2D[c], atol=1e-8)
    for end, hg, s in REF_RAY_2D:
        ray = O.raytrace(ax, tg[0], [end], np.zeros(2), 1.0, default_max_step(tt.shape[1:], (1,) * 2, 1.0), hg)[0]
        assert np.allclose(ray.sum(), s, atol=1e-8)
    tt, tg, vz = O.solve2d(np.ones((16, 16)), (1.0, 1.0), [[3.5, 3.5]], 2, True)
    for c in range(2):
        g = O.interp(ax, tg[0][..., c], [[0.0, 0.0]], stride=2)
        assert np.allclose(g, REF_GRAD_2D_SRC35[c], atol=1e-8)


@pytest.mark.parametrize("case", [REF_MESHIO_2D, REF_MESHIO_3D])
def test_known_answer_meshio_sums(case):
    nd = len(case["shape"])
    solve = O.solve3d if nd == 3 else O.solve2d
    tt, tg, vz = solve(np.ones(case["shape"]), (1.0,) * nd, [case["source"]], 2, True)
    assert np.allclose(tt[0].sum(), case["tt_sum"], atol=1e-8)
    flat = tg[0].reshape(-1, nd)
    assert np.all(flat[flat.shape[0] // 2] == 0.0)
    assert np.allclose(flat.sum(axis=0), 0.0)
    ax = model_axes(tt.shape[1:], (1.0,) * nd, np.zeros(nd))
    ray = O.raytrace(ax, tg[0], [np.zeros(nd)], np.array(case["source"]), 1.0,
                     default_max_step(tt.shape[1:], (1,) * nd, 1.0), True)[0]
    assert len(ray) == case["ray_len"]


def _solve(g, nd, sources=None, nsweep=None):
    solve = O.solve3d if nd == 3 else O.solve2d
    src = g["sources"] if sources is None else sources
    return solve(1.0 / g["velocity"], g["gridsize"], src - g["origin"],
                 int(g["nsweep"]) if nsweep is None else nsweep, True)


@pytest.mark.parametrize("nd", [2, 3])
def test_golden_solve(nd, golden2d, golden3d):
    g = golden3d if nd == 3 else golden2d
    tt, tg, vz = _solve(g, nd)
    assert max_rel(tt, g["tt"]) <= TOL_ORACLE_VS_REF
    assert np.abs(tg - g["ttgrad"]).max() <= 1e-12
    assert np.array_equal(vz, g["vzero"])
    if nd == 3:
        tt1, tg1, _ = _solve(g, nd, g["sources"][:1], 1)
        assert max_rel(tt1[0], g["tt_nsweep1"]) <= TOL_ORACLE_VS_REF
        assert np.abs(tg1[0] - g["ttgrad_nsweep1"]).max() <= 1e-12
    else:
        tt3, tg3, _ = _solve(g, nd, g["sources"][:2], 3)
        assert max_rel(tt3, g["tt_nsweep3"]) <= TOL_ORACLE_VS_REF
        assert np.abs(tg3 - g["ttgrad_nsweep3"]).max() <= 1e-12


@pytest.mark.parametrize("nd", [2, 3])
def test_golden_interp_and_rays(nd, golden2d, golden3d):
    g = golden3d if nd == 3 else golden2d
    tt, tg, vz = _solve(g, nd)
    ax = model_axes(tt.shape[1:], g["gridsize"], g["origin"])
    for s in range(len(g["sources"])):
        got = O.vinterp(ax, tt[s], g["points"], g["sources"][s], vz[s])
        assert max_rel(got, g["vinterp"][s]) <= TOL_ORACLE_VS_REF
        for c in range(nd):
            gi = O.interp(ax, tg[s][..., c], g["points"], stride=nd)
            assert np.array_equal(np.isnan(gi), np.isnan(g["gradinterp"][s][c]))
            assert np.nanmax(np.abs(gi - g["gradinterp"][s][c])) <= 1e-12
        stepsize = float(min(g["gridsize"]))
        ms = default_max_step(tt.shape[1:], g["gridsize"], stepsize)
        for hg in (0, 1):
            rays = O.raytrace(ax, tg[s], g["receivers"], g["sources"][s], stepsize, ms, hg)
            assert np.array_equal([len(r) for r in rays], g[f"raylen_s{s}_hg{hg}"])
            assert np.abs(np.concatenate(rays) - g[f"rays_s{s}_hg{hg}"]).max() <= 1e-9
    vel_ax = model_axes(g["velocity"].shape, g["gridsize"], g["origin"])
    vi = O.interp(vel_ax, g["velocity"], g["points"])
    assert max_rel(vi, g["velinterp"]) == 0.0


def test_source_out_of_bound_raises():
    with pytest.raises(ValueError, match="source out of bound"):
        O.solve3d(np.ones((4, 4, 4)), (1.0, 1.0, 1.0), [[5.0, 0.0, 0.0]])
    with pytest.raises(ValueError, match="source out of bound"):
        O.solve2d(np.ones((4, 4)), (1.0, 1.0), [[-0.1, 0.0]])


def test_ray_errors():
    tt, tg, vz = O.solve3d(np.ones((6, 6, 6)), (1.0, 1.0, 1.0), [[0.0, 0.0, 0.0]], 2, True)
    ax = model_axes(tt.shape[1:], (1.0,) * 3, np.zeros(3))
    with pytest.raises(ValueError, match="end point out of bound"):
        O.raytrace(ax, tg[0], [[7.0, 0.0, 0.0]], np.zeros(3), 1.0, 100)
    with pytest.raises(RuntimeError, match="maximum number of steps reached"):
        O.raytrace(ax, tg[0], [[6.0, 6.0, 6.0]], np.zeros(3), 0.1, 5)
