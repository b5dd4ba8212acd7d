"""Shared cases of the adjoint tests: small seeded tomography problems and the
finite-difference derivative of the oracle's receiver-traveltime loss."""

import numpy as np

from oracle import oracle as O

D = (10.0, 10.0, 10.0)


def velocity(shape, anomaly, seed=0, perturb=True):
    """Layered model, optionally with a Gaussian anomaly, times a seeded +-2 %
    cell perturbation when ``perturb``. The perturbation keeps every slowness
    distinct: the operators take the minimum slowness of 2 or 4 cells, and at
    an exact tie the solver has only one-sided derivatives."""
    nz, nx, ny = shape
    z = (np.arange(nz) + 0.5) * D[0]
    rng = np.random.default_rng(seed)
    v = (1600.0 + 0.8 * z)[:, None, None] * (1.0 + 0.02 * perturb * rng.uniform(-1.0, 1.0, shape))
    if anomaly:
        c = np.array(shape) * np.array(D) * np.array([0.5, 0.45, 0.55])
        zz, xx, yy = np.meshgrid(
            *[(np.arange(n) + 0.5) * h for n, h in zip(shape, D)], indexing="ij"
        )
        r2 = (zz - c[0]) ** 2 + (xx - c[1]) ** 2 + (yy - c[2]) ** 2
        v *= 1.0 + 0.08 * np.exp(-r2 / (2.0 * 30.0**2))
    return v


def geometry(shape, nsrc, nrec, seed):
    """Seeded off-grid surface sources and receivers."""
    rng = np.random.default_rng(seed)
    ext = np.array(shape) * np.array(D)
    src = np.column_stack(
        [np.zeros(nsrc), rng.uniform(0.1, 0.9, nsrc) * ext[1], rng.uniform(0.1, 0.9, nsrc) * ext[2]]
    )
    rec = np.column_stack(
        [np.zeros(nrec), rng.uniform(0.0, 1.0, nrec) * ext[1], rng.uniform(0.0, 1.0, nrec) * ext[2]]
    )
    return src, rec


def oracle_times(v, src, rec, nsweep):
    """[nsrc, nrec] apparent-velocity traveltimes through the oracle."""
    tt, _, vz = O.solve3d(1.0 / v, D, src, nsweep, False)
    ax = O.axes(tt.shape[1:], D, np.zeros(3))
    return np.stack([O.vinterp(ax, tt[s], rec, src[s], vz[s]) for s in range(len(src))])


def oracle_velocity_gradient(v, src, rec, nsweep, t_obs):
    """d(0.5 sum (T - t_obs)^2)/d(velocity) from the oracle's adjoint."""
    T = oracle_times(v, src, rec, nsweep)
    s = 1.0 / v
    return -O.adjoint3d(s, D, src, nsweep, rec, T - t_obs) * s * s


def central_difference(v, idx, rel, src, rec, nsweep, t_obs):
    """Central difference of the loss in velocity cell ``idx`` with step
    ``rel * v[idx]``. L(v+h) - L(v-h) is summed term by term as
    0.5 (tp - tm)(tp + tm - 2 t_obs), so no two nearly equal losses are
    subtracted."""
    h = rel * v[idx]
    vp = v.copy()
    vp[idx] += h
    vm = v.copy()
    vm[idx] -= h
    tp, tm = oracle_times(vp, src, rec, nsweep), oracle_times(vm, src, rec, nsweep)
    return float(np.sum(0.5 * (tp - tm) * (tp + tm - 2.0 * t_obs))) / (2.0 * h)


def check_cells(g, nbig=30, nrand=20, seed=5):
    """The largest-gradient cells and a seeded sample of the others."""
    rng = np.random.default_rng(seed)
    flat = np.abs(g).ravel()
    big = np.argsort(flat)[::-1][:nbig]
    rest = np.setdiff1d(np.flatnonzero(flat > 0), big)
    return np.concatenate([big, rng.choice(rest, nrand, replace=False)])
