"""Pin the CPU oracle on the benchmark workloads' own model recipes (CPU only).

``tests/golden/golden_configs.npz`` holds the reference's results (imported
from its source tree by ``tests/golden/make_golden_configs.py``) on the plain
2D workload at its full size and on reduced grids of the 3D recipes. The inputs
are rebuilt here from the same seeded builders in ``bench.py``; their digests
confirm they are the inputs the reference saw.
"""

import hashlib
import os
import sys

import numpy as np
import pytest

from helpers import max_rel

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytest.importorskip("scipy")

# The oracle restates `x ** 0.5` and `x ** 2.0` as sqrt and x*x where the
# pure-Python reference calls pow(); they differ in the last bit on a few 3D
# nodes. The 2D solve is bit-identical.
TOL = 1e-13


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden_configs.npz")))


def digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def test_plain_2d_workload_full_size_bitwise(gold):
    v, v0, src, d = bench.config1_models()
    assert np.array_equal(digest(v), gold["c1_v_digest"])
    assert np.array_equal(digest(v0), gold["c1_v0_digest"])
    t = O.solve2d(1.0 / v, d, [src], 2, False)[0][0]
    t0 = O.solve2d(1.0 / v0, d, [src], 2, False)[0][0]
    assert np.array_equal(digest(t), gold["c1_tt_digest"])
    assert np.array_equal(digest(t0), gold["c1_tt0_digest"])
    assert np.array_equal(t[::10, ::10], gold["c1_tt_sample"])
    # the reference's discretisation error on the noise-free v(z) model
    ta, far = bench.linear_gradient_times(v0.shape, d, src)
    rel = np.abs(t0 - ta)[far] / ta[far]
    # (numpy's arccosh may differ in the last bit between hosts)
    assert abs(rel.max() / gold["c1_analytic_rel_max"] - 1.0) <= 1e-9
    assert abs(np.median(rel) / gold["c1_analytic_rel_median"] - 1.0) <= 1e-9


def test_layered_3d_recipe(gold):
    shape = (24, 32, 40)
    v = bench.layered_model(shape)
    assert np.array_equal(digest(v), gold["c3_v_digest"])
    src, rec = gold["c3_src"], gold["c3_rec"]
    assert np.array_equal(src, bench.surface_sources(shape, n_side=2))
    tt, tg, vz = O.solve3d(1.0 / v, bench.D, src, 2, True)
    assert max_rel(tt.sum(axis=(1, 2, 3)), gold["c3_tt_sum"]) <= TOL
    assert max_rel(tt[:, ::3, ::3, ::3], gold["c3_tt_sample"]) <= TOL
    assert np.abs(tg[:, ::5, ::5, ::5] - gold["c3_grad_sample"]).max() <= 1e-10
    assert np.abs(tg.sum(axis=(1, 2, 3)) - gold["c3_grad_sum"]).max() <= 1e-8
    assert np.array_equal(vz, gold["c3_vzero"])
    ax = O.axes(tt.shape[1:], bench.D, np.zeros(3))
    picks = np.stack([O.vinterp(ax, tt[s], rec, src[s], vz[s]) for s in range(len(src))])
    assert max_rel(picks, gold["c3_picks"]) <= TOL
    max_step = int(2.0 * sum((n * h) ** 2 for n, h in zip(tt.shape[1:], bench.D)) ** 0.5 / 10.0)
    rays = [r for s in range(len(src))
            for r in O.raytrace(ax, tg[s], rec[:6], src[s], 10.0, max_step, False)]
    assert np.array_equal([len(r) for r in rays], gold["c3_raylen"])
    assert np.abs(np.concatenate(rays) - gold["c3_rays"]).max() <= 1e-9


def test_uneven_batch_recipe(gold):
    for m, (v, d, s) in enumerate(bench.uneven_models(2, seed=48, sizes=(16, 28))):
        assert np.array_equal(digest(v), gold[f"c4_m{m}_v_digest"])
        tt = O.solve3d(1.0 / v, d, s, 2, False)[0]
        assert max_rel(tt.sum(axis=(1, 2, 3)), gold[f"c4_m{m}_tt_sum"]) <= TOL
        assert max_rel(tt[:, ::2, ::3, ::2], gold[f"c4_m{m}_tt_sample"]) <= TOL
