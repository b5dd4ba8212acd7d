"""The oracle's adjoint of the 3D solve (CPU only) against central finite
differences of the oracle's own solve and receiver interpolation.

The oracle's solve is pinned to the reference; its adjoint is the checker of
the CUDA adjoint, so it is pinned here by differences taken through that
solve, with the loss 0.5 * sum((T - T_obs)^2) over source-receiver pairs.
"""

import numpy as np
import pytest

from adjoint_cases import (
    central_difference,
    check_cells,
    geometry,
    oracle_times,
    oracle_velocity_gradient,
    velocity,
)

SHAPE = (12, 14, 16)


def _case(nsweep, perturb):
    src, rec = geometry(SHAPE, 3, 24, 1)
    t_obs = oracle_times(velocity(SHAPE, True, perturb=perturb), src, rec, nsweep)
    v0 = velocity(SHAPE, False, perturb=perturb)
    g = oracle_velocity_gradient(v0, src, rec, nsweep, t_obs)
    return src, rec, t_obs, v0, g


@pytest.mark.parametrize("nsweep", [1, 2, 4])
def test_oracle_adjoint_matches_finite_differences(nsweep):
    """Every slowness distinct: the solve is differentiable at the model, and
    the adjoint matches central differences (relative step 1e-6) to 1e-6."""
    src, rec, t_obs, v0, g = _case(nsweep, True)
    gmax = np.abs(g).max()
    bad = []
    for c in check_cells(g):
        idx = np.unravel_index(c, SHAPE)
        fd = central_difference(v0, idx, 1e-6, src, rec, nsweep, t_obs)
        # the absolute floor covers the rounding of the differences on cells
        # whose derivative is ~1e-10 of the largest
        if abs(fd - g[idx]) > 1e-6 * abs(fd) + 1e-10 * gmax:
            bad.append((idx, g[idx], fd))
    assert not bad, bad


def test_oracle_adjoint_at_tied_slowness_is_the_central_derivative():
    """Pure layered model: the 2- and 4-cell slowness minima of the operators
    tie at almost every node, where the solve has different left and right
    derivatives. The adjoint gives each tied cell the mean of the two, the
    limit of central differences; at a finite step h those carry an O(h) bias
    (the two sides curve differently), so the error shrinks with the step."""
    nsweep = 2
    src, rec, t_obs, v0, g = _case(nsweep, False)
    gmax = np.abs(g).max()
    cells = check_cells(g, 12, 0)
    err = {}
    for rel in (1e-4, 1e-6):
        e = []
        for c in cells:
            idx = np.unravel_index(c, SHAPE)
            fd = central_difference(v0, idx, rel, src, rec, nsweep, t_obs)
            e.append(abs(fd - g[idx]) / (abs(fd) + 1e-10 * gmax))
        err[rel] = np.array(e)
    assert err[1e-6].max() < 2e-5
    # first-order convergence in the step on the cells with a visible bias
    sel = err[1e-4] > 1e-4
    assert sel.any()
    assert np.all(err[1e-6][sel] < 0.05 * err[1e-4][sel])
