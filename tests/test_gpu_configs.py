"""Every benchmark workload at its stated size, on the GPU against the oracle.

The workloads are built by the same seeded builders as ``bench.py``:

1. plain 2D: 200 x 300 noisy v(z), one off-grid source, nsweep=2, both 2D
   kernels; and the noise-free v(z) model against the analytic
   linear-gradient traveltime (the reference's own discretisation error);
2. plain 3D: 150 x 200 x 200 layered, one surface source with gradients,
   10,000 traveltime queries and 400 rays;
3. batched 3D: 256 sources on 128 x 256 x 256 with gradients (the timed team
   kernel and its gradient post-pass; traveltime offsets past 2^31 elements,
   gradient offsets past 6 * 2^30), checked on sampled sources including the
   last one, with their picks and rays, and the batched ray kernel;
4. uneven batch: 64 models of 32-160 cells per axis, 1-16 sources each, in one
   launch, against one solve per model and the oracle on a sample;
5. adjoint: 96 x 128 x 128, 64 sources x 400 receivers: the forward picks and
   the velocity gradient against the oracle's forward and reverse-mode
   adjoint, on every cell.

Everything but the adjoint is compared bit for bit; the adjoint's partials
have no bitwise counterpart (they may contract and use reciprocals), so it is
compared to 1e-12 of its largest entry.
"""

import os
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402
import fteikpy_gb300 as fp  # noqa: E402
from fteikpy_gb300 import _device, _lib, _solver  # noqa: E402
from fteikpy_gb300._grid import trace_rays_device  # noqa: E402
from oracle import oracle as O  # noqa: E402

# The measured discretisation error of the reference's 2D solve on the
# noise-free v(z) model against the analytic linear-gradient traveltime, nodes
# farther than 5 cells from the source (max 2.219e-3, median 8.480e-5).
C1_ANALYTIC_MAX, C1_ANALYTIC_MEDIAN = 2.22e-3, 8.49e-5


def _need(gb):
    free, _ = torch.cuda.mem_get_info()
    if free < gb * 1e9:
        pytest.skip(f"needs about {gb} GB of free device memory")


def _max_step(shape, d):
    return int(2.0 * sum((n * h) ** 2 for n, h in zip(shape, d)) ** 0.5 / min(d))


def test_config1_plain_2d_both_kernels_and_analytic():
    lib = _lib.load()
    v, v0, src, d = bench.config1_models()
    ref = O.solve2d(1.0 / v, d, [src], 2, False)[0][0]
    try:
        # a block and a warp per source, each with and without speculated
        # updates, one thread per source; integer-key and IEEE comparisons
        for warp, spec in ((2, -1), (2, 0), (1, -1), (1, 0), (0, -1)):
            for keys in (-1, 0):
                assert lib.fteik_set_option(b"sweep2d_warp", warp) == _lib.OK
                assert lib.fteik_set_option(b"sweep2d_speculate", spec) == _lib.OK
                assert lib.fteik_set_option(b"sweep2d_keys", keys) == _lib.OK
                got = fp.Eikonal2D(v, d).solve(src, nsweep=2).grid
                assert np.array_equal(got, ref), (warp, spec, keys)
    finally:
        for name in (b"sweep2d_warp", b"sweep2d_speculate", b"sweep2d_keys"):
            lib.fteik_set_option(name, -1)
    t0 = fp.Eikonal2D(v0, d).solve(src, nsweep=2).grid
    assert np.array_equal(t0, O.solve2d(1.0 / v0, d, [src], 2, False)[0][0])
    ta, far = bench.linear_gradient_times(v0.shape, d, src)
    rel = np.abs(t0 - ta)[far] / ta[far]
    assert rel.max() <= C1_ANALYTIC_MAX and np.median(rel) <= C1_ANALYTIC_MEDIAN


def test_config2_plain_3d_queries_and_rays():
    shape = (150, 200, 200)
    v = bench.layered_model(shape)
    rng = np.random.default_rng(2)
    ext = np.array(shape) * np.array(bench.D)
    src = np.array([0.0, rng.uniform(0.2, 0.8) * ext[1], rng.uniform(0.2, 0.8) * ext[2]])
    pts = rng.uniform([0.0, 0.0, 0.0], ext, (10000, 3))
    rec = np.column_stack([np.zeros(400), rng.uniform(0, ext[1], 400),
                           rng.uniform(0, ext[2], 400)])
    tt = fp.Eikonal3D(v, bench.D).solve(src, nsweep=2, return_gradient=True)
    tto, tgo, vzo = O.solve3d(1.0 / v, bench.D, [src], 2, True)
    assert np.array_equal(tt.grid, tto[0])
    assert np.array_equal(tt.gradient_tensor.cpu().numpy(), tgo[0])
    ax = O.axes(tto.shape[1:], bench.D, np.zeros(3))
    assert np.array_equal(tt(pts), O.vinterp(ax, tto[0], pts, src, vzo[0]))
    rays = tt.raytrace(rec)
    ref = O.raytrace(ax, tgo[0], rec, src, 10.0, _max_step(tto.shape[1:], bench.D), False)
    assert len(rays) == len(ref)
    for a, b in zip(rays, ref):
        assert np.array_equal(a, b)


def test_config3_batch_with_gradients_full_size():
    _need(90)
    lib = _lib.load()
    v = bench.layered_model()
    src = bench.surface_sources()
    rec = bench.surface_receivers()
    assert len(src) == 256
    eik = fp.Eikonal3D(v, bench.D)
    tts = eik.solve(src, nsweep=2, return_gradient=True)
    assert lib.fteik_last_sweep_kernel() == b"sweep3d_team_kernel"
    # every result is a view of the solve's own device memory
    nodes = int(np.prod(np.array(bench.SHAPE) + 1))
    assert tts[255].tensor.data_ptr() == tts[0].tensor.data_ptr() + 255 * nodes * 8
    assert tts[255].gradient_tensor.data_ptr() == (
        tts[0].gradient_tensor.data_ptr() + 255 * nodes * 3 * 8)
    picked = [0, 97, 255]
    tto, tgo, vzo = O.solve3d(1.0 / v, bench.D, src[picked], 2, True, nthreads=len(picked))
    ax = O.axes(tto.shape[1:], bench.D, np.zeros(3))
    ms = _max_step(tto.shape[1:], bench.D)
    for q, s in enumerate(picked):
        assert torch.equal(tts[s].tensor.cpu(), torch.from_numpy(tto[q])), s
        assert torch.equal(tts[s].gradient_tensor.cpu(), torch.from_numpy(tgo[q])), s
        assert tts[s]._vzero == vzo[q]
        assert np.array_equal(tts[s](rec), O.vinterp(ax, tto[q], rec, src[s], vzo[q]))
        rays = tts[s].raytrace(rec)
        ref = O.raytrace(ax, tgo[q], rec, src[s], 10.0, ms, False)
        assert all(np.array_equal(a, b) for a, b in zip(rays, ref)), s
    # the batched ray kernel over all 256 gradient grids, nodes * 3 elements
    # apart from the first one's (as the benchmark runs it)
    axes = [_device.to_device(a) for a in ax]
    gidx = torch.arange(256, dtype=torch.int32, device=axes[0].device).repeat_interleave(400)
    ends = _device.to_device(np.tile(rec, (256, 1)))
    packed, lengths = trace_rays_device(3, axes, tts[0].gradient_tensor, gidx, ends,
                                        _device.to_device(src), 10.0, ms, False, nodes * 3)
    off = np.concatenate([[0], np.cumsum(lengths.cpu().numpy())])
    last = packed[off[255 * 400]:].cpu().numpy()
    ref = O.raytrace(ax, tgo[2], rec, src[255], 10.0, ms, False)
    for r in range(400):
        a, b = off[255 * 400 + r] - off[255 * 400], off[255 * 400 + r + 1] - off[255 * 400]
        assert np.array_equal(last[a:b], ref[r]), r
    # a single-source solve (one warp per pencil, another schedule) equals the batch
    slow = eik._device_slowness()
    del tts, packed
    for s in (0, 255):
        one, _, _ = _solver.solve3d_device(slow, bench.D, src[s:s + 1], 2, False)
        assert np.array_equal(one[0].cpu().numpy(), tto[picked.index(s)])


def test_config4_uneven_models_one_launch():
    cases = bench.uneven_models()
    solvers = [fp.Eikonal3D(v, d) for v, d, _ in cases]
    sources = [s for _, _, s in cases]
    out = fp.solve_batch(solvers, sources, nsweep=2)
    for m, (eik, s) in enumerate(zip(solvers, sources)):
        one = eik.solve(s, nsweep=2)
        for a, b in zip(out[m], one):
            assert torch.equal(a.tensor.view(torch.int64), b.tensor.view(torch.int64)), m
            assert a._vzero == b._vzero
    for m in range(0, len(cases), 16):
        v, d, s = cases[m]
        ref = O.solve3d(1.0 / v, d, s, 2, False)[0]
        assert np.array_equal(np.stack([t.grid for t in out[m]]), ref), m


def test_config5_adjoint_full_size():
    _need(40)
    shape = (96, 128, 128)
    v0, vt = bench.tomography_models(shape)
    src = bench.surface_sources(shape, n_side=8, seed=7)
    rec = bench.surface_receivers(shape, n=400, seed=11)
    dev = torch.device("cuda", torch.cuda.current_device())
    t_obs = fp.traveltimes(torch.tensor(vt, device=dev), bench.D, src, rec, 2).detach()
    vel = torch.tensor(v0, device=dev, requires_grad=True)
    T = fp.traveltimes(vel, bench.D, src, rec, 2)
    (0.5 * ((T - t_obs) ** 2).sum()).backward()
    g = vel.grad.cpu().numpy()

    tt, _, vz = O.solve3d(1.0 / v0, bench.D, src, 2, False)
    ax = O.axes(tt.shape[1:], bench.D, np.zeros(3))
    t_ref = np.stack([O.vinterp(ax, tt[s], rec, src[s], vz[s]) for s in range(len(src))])
    assert np.array_equal(T.detach().cpu().numpy(), t_ref)
    s0 = 1.0 / v0
    resid = t_ref - t_obs.cpu().numpy()
    g_ref = -O.adjoint3d(s0, bench.D, src, 2, rec, resid) * s0 * s0
    assert np.abs(g - g_ref).max() <= 1e-12 * np.abs(g_ref).max()
    # the start model is a linear gradient: the 3D solve equals the oracle bit
    # for bit, so its error against the analytic traveltime is the reference's
    # own discretisation error (oracle: max 6.9e-2, median 1.08e-3 relative,
    # nodes farther than 5 cells from the source)
    one = fp.Eikonal3D(v0, bench.D).solve(src[0], nsweep=2).grid
    assert np.array_equal(one, tt[0])
    ta, far = bench.linear_gradient_times(shape, bench.D, src[0])
    rel = np.abs(one - ta)[far] / ta[far]
    assert rel.max() < 0.07 and np.median(rel) < 1.1e-3
