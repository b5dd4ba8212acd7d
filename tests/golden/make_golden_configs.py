"""Generate ``golden_configs.npz``: the reference's results on the benchmark
workloads' own model recipes, from the fteikpy reference itself.

Run once, in a container where the reference source tree is available:

    python tests/golden/make_golden_configs.py /path/to/fteikpy-reference

The reference is imported in pure-Python mode through the numba stand-in under
``oracle/numba_shim`` (the mode of the reference's own CI,
``NUMBA_DISABLE_JIT=1``), about 20 us per 3D node update, so the 3D cases are
reduced grids of the same recipes. The inputs come from the model builders in
``bench.py`` (seeded); the fixture keeps SHA-256 digests of them, so a test
can confirm it rebuilt the same inputs, and of the outputs where the oracle is
expected to be bit-identical (2D), plus sums and strided samples of every
output.

Cases:

* ``c1_*``: the plain 2D workload at its full size (200 x 300 cells at 10 m,
  noisy v(z), source (5.3, 1234.7), nsweep=2), and the same solve on the
  noise-free v(z) model, whose error against the analytic linear-gradient
  traveltime is the reference's own discretisation error.
* ``c3_*``: the layered model of the 3D workloads on 24 x 32 x 40 cells, the
  2 x 2 jittered surface sources, nsweep=2 with gradients, the picks at 50
  surface receivers, and rays to 6 of them from each source.
* ``c4_*``: two models of the uneven-batch recipe (sizes drawn from [16, 28]
  instead of [32, 160]), every source, nsweep=2.
"""

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def main(ref_path):
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "oracle", "numba_shim"))
    sys.path.insert(0, ref_path)
    import fteikpy

    import bench

    out = {}
    # ---------------- plain 2D workload, full size ----------------
    v, v0, src, d = bench.config1_models()
    t = fteikpy.Eikonal2D(v, d).solve(src, nsweep=2).grid
    t0 = fteikpy.Eikonal2D(v0, d).solve(src, nsweep=2).grid
    ta, far = bench.linear_gradient_times(v0.shape, d, src)
    rel = np.abs(t0 - ta)[far] / ta[far]
    out.update(
        c1_v_digest=digest(v), c1_v0_digest=digest(v0),
        c1_tt_digest=digest(t), c1_tt_sum=t.sum(), c1_tt_sample=t[::10, ::10],
        c1_tt0_digest=digest(t0), c1_tt0_sum=t0.sum(), c1_tt0_sample=t0[::10, ::10],
        c1_analytic_rel_max=rel.max(), c1_analytic_rel_median=np.median(rel),
    )
    # ---------------- layered 3D recipe, reduced grid ----------------
    shape = (24, 32, 40)
    v = bench.layered_model(shape)
    src = bench.surface_sources(shape, n_side=2)
    rec = bench.surface_receivers(shape, n=50, seed=11)
    tts = fteikpy.Eikonal3D(v, bench.D).solve(src, nsweep=2, return_gradient=True)
    tt = np.stack([x.grid for x in tts])
    tg = np.stack([x._gradient for x in tts])
    rays, lens = [], []
    for x in tts:
        for r in x.raytrace(rec[:6]):
            rays.append(r)
            lens.append(len(r))
    out.update(
        c3_v_digest=digest(v), c3_src=src, c3_rec=rec,
        c3_tt_sum=tt.sum(axis=(1, 2, 3)), c3_tt_sample=tt[:, ::3, ::3, ::3],
        c3_grad_sum=tg.sum(axis=(1, 2, 3)), c3_grad_sample=tg[:, ::5, ::5, ::5],
        c3_vzero=np.array([x._vzero for x in tts]),
        c3_picks=np.stack([x(rec) for x in tts]),
        c3_rays=np.concatenate(rays), c3_raylen=np.array(lens),
    )
    # ---------------- uneven-batch recipe, reduced sizes ----------------
    for m, (v, d, s) in enumerate(bench.uneven_models(2, seed=48, sizes=(16, 28))):
        tts = fteikpy.Eikonal3D(v, d).solve(s, nsweep=2)
        tt = np.stack([x.grid for x in tts])
        out[f"c4_m{m}_v_digest"] = digest(v)
        out[f"c4_m{m}_tt_sum"] = tt.sum(axis=(1, 2, 3))
        out[f"c4_m{m}_tt_sample"] = tt[:, ::2, ::3, ::2]
    np.savez_compressed(os.path.join(HERE, "golden_configs.npz"), **out)
    print("wrote golden_configs.npz")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
