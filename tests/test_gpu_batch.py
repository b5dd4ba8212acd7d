"""Launch shapes, the multi-model batch and the autotuner of the 3D solve
against the oracle: every shape and every batch gives the reference's bits."""

import numpy as np
import pytest

import fteikpy_gb300 as fp
from fteikpy_gb300 import _lib
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def bitwise(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def gradient_model(shape, d, seed):
    """Linear-gradient velocity with seeded +-10 % cell noise."""
    rng = np.random.default_rng(seed)
    z = (np.arange(shape[0]) + 0.5) * d[0]
    v = (1500.0 + 0.7 * z)[:, None, None] * np.ones(shape)
    return v * (1.0 + 0.1 * rng.uniform(-1.0, 1.0, shape))


def sources_in(rng, shape, d, n):
    ext = np.array(shape) * np.array(d)
    return rng.uniform(0.0, 1.0, (n, 3)) * ext


@pytest.fixture
def options():
    lib = _lib.load()
    yield lib
    for name in (b"sweep_pencil", b"sweep_chunk", b"sweep_coef", b"sweep_keep_test",
                 b"sweep_team"):
        lib.fteik_set_option(name, -1)
    lib.fteik_clear_tuning()


@pytest.mark.parametrize("pencil", [2, 4, 8])
@pytest.mark.parametrize("chunk", [1, 4, 32])
@pytest.mark.parametrize("coef", [0, 1])
@pytest.mark.parametrize("team", [0, 1])
def test_every_launch_shape_gives_the_reference_bits(options, pencil, chunk, coef, team):
    lib = options
    assert lib.fteik_set_option(b"sweep_pencil", pencil) == 0
    assert lib.fteik_set_option(b"sweep_chunk", chunk) == 0
    assert lib.fteik_set_option(b"sweep_coef", coef) == 0
    assert lib.fteik_set_option(b"sweep_team", team) == 0
    rng = np.random.default_rng(pencil * 100 + chunk * 10 + coef)
    shape, d = (17, 23, 37), (9.0, 11.0, 10.0)
    v = gradient_model(shape, d, 3)
    # 3 and 6 sources: the team kernel's last group of 4 has idle warps
    src = sources_in(rng, shape, d, 3 + 3 * team)
    tt_o, tg_o, _ = O.solve3d(1.0 / v, d, src, 2, True)
    tts = fp.Eikonal3D(v, d).solve(src, nsweep=2, return_gradient=True)
    assert bitwise(np.stack([t.grid for t in tts]), tt_o)
    assert bitwise(np.stack([t._gradient.cpu().numpy() for t in tts]), tg_o)


def test_options_reject_unsupported_values(options):
    lib = options
    assert lib.fteik_set_option(b"sweep_pencil", 3) != 0
    assert lib.fteik_set_option(b"sweep_chunk", 6) != 0
    assert lib.fteik_set_option(b"sweep_chunk", 128) != 0
    import ctypes

    v = ctypes.c_longlong()
    assert lib.fteik_set_option(b"sweep_chunk", 8) == 0
    assert lib.fteik_get_option(b"sweep_chunk", ctypes.byref(v)) == 0 and v.value == 8


def uneven_batch(seed, nmodel, lo=8, hi=40):
    rng = np.random.default_rng(seed)
    solvers, sources, cases = [], [], []
    for _ in range(nmodel):
        shape = tuple(int(x) for x in rng.integers(lo, hi + 1, 3))
        d = tuple(float(x) for x in rng.uniform(5.0, 20.0, 3))
        v = gradient_model(shape, d, int(rng.integers(1 << 30)))
        src = sources_in(rng, shape, d, int(rng.integers(1, 5)))
        solvers.append(fp.Eikonal3D(v, d))
        sources.append(src)
        cases.append((v, d, src))
    return solvers, sources, cases


@pytest.mark.parametrize("grad", [False, True])
@pytest.mark.parametrize("pencil", [None, 2, 8])
def test_batch_of_uneven_models_equals_oracle(options, grad, pencil):
    if pencil:
        options.fteik_set_option(b"sweep_pencil", pencil)
    solvers, sources, cases = uneven_batch(11 + (pencil or 0), 7)
    out = fp.solve_batch(solvers, sources, nsweep=2, return_gradient=grad)
    assert len(out) == len(cases)
    for res, (v, d, src) in zip(out, cases):
        tt_o, tg_o, vz_o = O.solve3d(1.0 / v, d, src, 2, grad)
        assert bitwise(np.stack([t.grid for t in res]), tt_o)
        assert np.array_equal([t._vzero for t in res], vz_o)
        if grad:
            assert bitwise(np.stack([t._gradient.cpu().numpy() for t in res]), tg_o)


def test_batch_equals_one_solve_per_model_and_handles_single_sources():
    solvers, sources, cases = uneven_batch(5, 4)
    sources[1] = sources[1][0]  # a single source: one grid, as Eikonal3D.solve returns
    out = fp.solve_batch(solvers, sources, nsweep=1)
    assert isinstance(out[1], fp.TraveltimeGrid3D)
    for eik, src, res in zip(solvers, sources, out):
        ref = eik.solve(src, nsweep=1)
        if isinstance(ref, list):
            assert all(bitwise(a.grid, b.grid) for a, b in zip(ref, res))
        else:
            assert bitwise(ref.grid, res.grid)


def test_batch_source_out_of_bound_raises():
    solvers, sources, _ = uneven_batch(6, 2)
    sources[1] = np.vstack([sources[1], [[-1.0, 0.0, 0.0]]])
    with pytest.raises(ValueError):
        fp.solve_batch(solvers, sources)


def test_autotune_single_and_batch(options):
    rng = np.random.default_rng(8)
    shape, d = (24, 40, 36), (10.0, 10.0, 10.0)
    v = gradient_model(shape, d, 8)
    src = sources_in(rng, shape, d, 6)
    eik = fp.Eikonal3D(v, d)
    ref = np.stack([t.grid for t in eik.solve(src, nsweep=2)])
    best = fp.autotune(eik, src)
    assert best["pencil"] in (2, 4, 8) and best["chunk"] in (1, 2, 4, 8, 16, 32)
    assert best["coef"] in (0, 1) and best["team"] in (0, 1) and best["ms"] > 0
    assert bitwise(np.stack([t.grid for t in eik.solve(src, nsweep=2)]), ref)
    solvers, sources, cases = uneven_batch(9, 5)
    best = fp.autotune(solvers, sources)
    assert best["pencil"] in (2, 4, 8) and best["ms"] > 0
    out = fp.solve_batch(solvers, sources, nsweep=2)
    for res, (v, d, s) in zip(out, cases):
        assert bitwise(np.stack([t.grid for t in res]), O.solve3d(1.0 / v, d, s, 2, False)[0])


@pytest.mark.parametrize("grad", [False, True])
def test_unchanged_node_test_gives_the_same_bits(options, grad):
    """Equal spacings enable the test that skips the 2D/3D operators of nodes
    that provably keep their value: on and off give the same bits."""
    lib = options
    rng = np.random.default_rng(4)
    shape, d = (30, 41, 37), (10.0, 10.0, 10.0)
    v = gradient_model(shape, d, 4)
    v[12:, :, :] *= 1.8  # a strong interface: head waves, late changes
    src = sources_in(rng, shape, d, 9)
    src[:4, 0] = 0.0
    res = {}
    for on in (1, 0):
        assert lib.fteik_set_option(b"sweep_keep_test", on) == 0
        assert lib.fteik_set_option(b"sweep_team", 1) == 0
        tts = fp.Eikonal3D(v, d).solve(src, nsweep=3, return_gradient=grad)
        res[on] = (np.stack([t.grid for t in tts]),
                   np.stack([t._gradient.cpu().numpy() for t in tts]) if grad else None)
    assert bitwise(res[0][0], res[1][0])
    if grad:
        assert bitwise(res[0][1], res[1][1])
    assert bitwise(res[1][0], O.solve3d(1.0 / v, d, src, 3, False)[0])


@pytest.mark.parametrize("nsrc", [4, 9, 16])
def test_team_kernel_equals_warp_kernel_on_a_layered_model(options, nsrc):
    """Team and warp-per-pencil kernels on an equal-spacing layered model
    (the unchanged-node test active), with gradients: same bits, and the
    oracle's."""
    lib = options
    rng = np.random.default_rng(nsrc)
    shape, d = (33, 40, 29), (10.0, 10.0, 10.0)
    v = gradient_model(shape, d, nsrc)
    v[15:] *= 1.6
    src = sources_in(rng, shape, d, nsrc)
    src[: nsrc // 2, 0] = 0.0
    out = {}
    for team in (0, 1):
        lib.fteik_set_option(b"sweep_team", team)
        tts = fp.Eikonal3D(v, d).solve(src, nsweep=2, return_gradient=True)
        out[team] = (np.stack([t.grid for t in tts]),
                     np.stack([t._gradient.cpu().numpy() for t in tts]))
    assert bitwise(out[0][0], out[1][0]) and bitwise(out[0][1], out[1][1])
    tt_o, tg_o, _ = O.solve3d(1.0 / v, d, src, 2, True)
    assert bitwise(out[1][0], tt_o) and bitwise(out[1][1], tg_o)


def test_solve_sharded_on_the_visible_devices_equals_one_solve():
    """The source list split over the visible devices (one here) gives the
    single solve's results, in source order, bit for bit."""
    rng = np.random.default_rng(21)
    shape, d = (14, 18, 22), (10.0, 10.0, 10.0)
    v = 1500.0 + 40.0 * np.arange(shape[0])[:, None, None] * np.ones(shape)
    v *= 1.0 + 0.05 * rng.uniform(-1, 1, shape)
    src = np.column_stack([rng.uniform(0, 140, 5), rng.uniform(0, 180, 5), rng.uniform(0, 220, 5)])
    eik = fp.Eikonal3D(v, d)
    one = eik.solve(src, nsweep=2, return_gradient=True)
    out = fp.solve_sharded(eik, src, nsweep=2, return_gradient=True)
    assert len(out) == len(one)
    for a, b in zip(out, one):
        assert np.array_equal(a.grid, b.grid)
        assert np.array_equal(a.gradient_tensor.cpu().numpy(), b.gradient_tensor.cpu().numpy())
        assert np.array_equal(a.source, b.source)
