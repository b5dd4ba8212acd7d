"""Generate the golden fixtures in this directory from the fteikpy reference.

Run once, in a container where the reference source tree is available:

    python tests/golden/make_golden.py /path/to/fteikpy-reference

The reference is imported in pure-Python mode through the numba stand-in under
``oracle/numba_shim`` (the mode the reference's own CI uses,
``NUMBA_DISABLE_JIT=1``). Every input (velocity model, sources, query points,
receivers) is generated here from fixed seeds and saved next to the outputs, so
the tests need neither the reference nor this script at run time.

Cases (all float64):

* ``golden3d.npz`` - a layered, noisy 3D model with anisotropic spacing and a
  non-zero origin; three sources (off-grid interior, on-grid node, on the
  bottom/side boundary) solved as one batch with ``nsweep=2`` and gradients,
  plus ``nsweep=1`` for the first source (leaves unreached nodes at ``Big``);
  traveltime (apparent-velocity) interpolation, gradient-grid interpolation,
  velocity interpolation and ray tracing with and without ``honor_grid``.
* ``golden2d.npz`` - the same for a 2D model with four sources that exercise
  the reference's source classification (off-grid, on a node, on a grid line
  in one axis only, on the model boundary) and the near-source operators.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def smooth_noise(rng, shape, passes=3):
    """Seeded noise smoothed by repeated 3-point box filtering, scaled to [-1, 1]."""
    p = rng.standard_normal(shape)
    for _ in range(passes):
        for ax in range(len(shape)):
            p = (np.roll(p, 1, ax) + p + np.roll(p, -1, ax)) / 3.0
    p -= p.min()
    p /= p.max()
    return 2.0 * p - 1.0


def model3d(shape=(16, 18, 20), seed=3):
    rng = np.random.default_rng(seed)
    nz, nx, ny = shape
    v = np.empty(shape)
    tops = np.sort(rng.integers(1, nz, 3))
    vels = np.sort(rng.uniform(1500.0, 4500.0, 4))
    layer = np.searchsorted(tops, np.arange(nz), side="right")
    v[:] = vels[layer][:, None, None]
    v *= 1.0 + 0.05 * smooth_noise(rng, shape)
    return v


def model2d(shape=(24, 32), seed=5):
    rng = np.random.default_rng(seed)
    nz, nx = shape
    z = np.arange(nz)[:, None]
    v = 1500.0 + 40.0 * z + np.zeros((nz, nx))
    v *= 1.0 + 0.1 * smooth_noise(rng, shape)
    return v


def pack_rays(rays):
    rays = rays if isinstance(rays, list) else [rays]
    lengths = np.array([len(r) for r in rays], dtype=np.int64)
    return np.concatenate(rays, axis=0), lengths


def main(ref_path):
    sys.path.insert(0, os.path.join(REPO, "oracle", "numba_shim"))
    sys.path.insert(0, ref_path)
    import fteikpy

    # ---------------- 3D ----------------
    v3 = model3d()
    gs3 = (9.0, 11.0, 10.0)
    og3 = np.array([5.0, -20.0, 3.0])
    nz, nx, ny = v3.shape
    ext3 = og3 + np.array(gs3) * np.array(v3.shape)
    src3 = np.array(
        [
            [og3[0] + 23.7, og3[1] + 101.3, og3[2] + 77.9],  # off-grid interior
            [og3[0] + 9.0 * 4, og3[1] + 11.0 * 9, og3[2] + 10.0 * 3],  # on a node
            [ext3[0], og3[1] + 150.2, ext3[2]],  # bottom / side boundary
        ]
    )
    eik3 = fteikpy.Eikonal3D(v3, gs3, og3)
    tts = eik3.solve(src3, nsweep=2, return_gradient=True)
    tt1 = eik3.solve(src3[0], nsweep=1, return_gradient=True)

    rng = np.random.default_rng(11)
    lo = og3 - 5.0
    hi = og3 + np.array(gs3) * (np.array(v3.shape) - 1) + 5.0
    pts3 = rng.uniform(lo, hi, size=(64, 3))
    pts3[:4] = og3 + np.array(gs3) * np.array([[0, 0, 0], [3, 7, 2], [15, 17, 19], [5, 0, 19]])
    pts3[4] = src3[0] + np.array([1.0, -2.0, 0.5])  # inside the source cell
    node_ext = og3 + np.array(gs3) * np.array(v3.shape)
    pts3[5] = node_ext  # last traveltime node (edge cases of the interpolation)
    pts3[6] = [node_ext[0], og3[1] + 40.0, og3[2] + 55.5]

    rec3 = np.column_stack(
        [
            np.full(6, og3[0]),
            og3[1] + np.array([3.0, 40.0, 77.7, 150.0, 190.0, 10.0]),
            og3[2] + np.array([2.0, 150.0, 33.3, 90.0, 199.0, 60.0]),
        ]
    )
    rec3[5] = [og3[0] + 100.0, og3[1] + 120.0, og3[2] + 50.0]

    out3 = dict(
        velocity=v3,
        gridsize=np.array(gs3),
        origin=og3,
        sources=src3,
        nsweep=2,
        tt=np.stack([t.grid for t in tts]),
        ttgrad=np.stack([t._gradient for t in tts]),
        vzero=np.array([t._vzero for t in tts]),
        tt_nsweep1=tt1.grid,
        ttgrad_nsweep1=tt1._gradient,
        points=pts3,
        vinterp=np.stack([t(pts3) for t in tts]),
        gradinterp=np.stack([[g(pts3) for g in t.gradient] for t in tts]),
        velinterp=eik3(pts3),
        receivers=rec3,
    )
    for s, t in enumerate(tts):
        for hg in (False, True):
            r, n = pack_rays(t.raytrace(rec3, honor_grid=hg))
            out3[f"rays_s{s}_hg{int(hg)}"] = r
            out3[f"raylen_s{s}_hg{int(hg)}"] = n
    r, n = pack_rays(tts[0].raytrace(rec3, stepsize=4.0))
    out3["rays_s0_step4"] = r
    out3["raylen_s0_step4"] = n
    np.savez_compressed(os.path.join(HERE, "golden3d.npz"), **out3)

    # ---------------- 2D ----------------
    v2 = model2d()
    gs2 = (10.0, 8.0)
    og2 = np.array([3.0, -7.0])
    ext2 = og2 + np.array(gs2) * np.array(v2.shape)
    src2 = np.array(
        [
            [og2[0] + 53.3, og2[1] + 123.7],  # off-grid (near-source operators)
            [og2[0] + 10.0 * 7, og2[1] + 8.0 * 12],  # on a node
            [og2[0] + 10.0 * 12, og2[1] + 101.1],  # on a z grid line only
            [ext2[0], og2[1] + 8.0 * 31 + 3.5],  # on the bottom boundary
            [og2[0] + 0.0, og2[1] + 3.25],  # on the top boundary, off-grid in x
        ]
    )
    eik2 = fteikpy.Eikonal2D(v2, gs2, og2)
    tts2 = eik2.solve(src2, nsweep=2, return_gradient=True)
    tts2_n3 = eik2.solve(src2[:2], nsweep=3, return_gradient=True)

    rng = np.random.default_rng(13)
    lo = og2 - 5.0
    hi = og2 + np.array(gs2) * (np.array(v2.shape) - 1) + 5.0
    pts2 = rng.uniform(lo, hi, size=(64, 2))
    pts2[:3] = og2 + np.array(gs2) * np.array([[0, 0], [23, 31], [4, 9]])
    pts2[3] = src2[0] + np.array([1.0, 2.0])
    pts2[4] = og2 + np.array(gs2) * np.array(v2.shape)
    pts2[5] = [og2[0] + 55.5, og2[1] + np.array(gs2[1]) * v2.shape[1]]

    rec2 = np.column_stack(
        [np.full(6, og2[0]), og2[1] + np.array([0.0, 20.0, 57.7, 150.0, 255.0, 201.0])]
    )
    rec2[5] = [og2[0] + 150.0, og2[1] + 30.0]

    out2 = dict(
        velocity=v2,
        gridsize=np.array(gs2),
        origin=og2,
        sources=src2,
        nsweep=2,
        tt=np.stack([t.grid for t in tts2]),
        ttgrad=np.stack([t._gradient for t in tts2]),
        vzero=np.array([t._vzero for t in tts2]),
        tt_nsweep3=np.stack([t.grid for t in tts2_n3]),
        ttgrad_nsweep3=np.stack([t._gradient for t in tts2_n3]),
        points=pts2,
        vinterp=np.stack([t(pts2) for t in tts2]),
        gradinterp=np.stack([[g(pts2) for g in t.gradient] for t in tts2]),
        velinterp=eik2(pts2),
        receivers=rec2,
    )
    for s, t in enumerate(tts2):
        for hg in (False, True):
            r, n = pack_rays(t.raytrace(rec2, honor_grid=hg))
            out2[f"rays_s{s}_hg{int(hg)}"] = r
            out2[f"raylen_s{s}_hg{int(hg)}"] = n
    r, n = pack_rays(tts2[0].raytrace(rec2, stepsize=3.0))
    out2["rays_s0_step3"] = r
    out2["raylen_s0_step3"] = n
    np.savez_compressed(os.path.join(HERE, "golden2d.npz"), **out2)
    print("wrote golden3d.npz and golden2d.npz")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
