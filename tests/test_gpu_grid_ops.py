"""Resample and smooth on the device against SciPy, which the reference calls
(fteikpy/_base.py:81-123, 165-212), and the reference's own known answers for
them (tests/test_eikonal3d.py:48-60, tests/test_eikonal2d.py:36-48)."""

import numpy as np
import pytest
from scipy.interpolate import RegularGridInterpolator
from scipy.ndimage import gaussian_filter

import fteikpy_gb300 as fp

pytestmark = pytest.mark.gpu


def scipy_resample(v, gridsize, origin, new_shape, method):
    axes = [o + h * np.arange(n) for o, h, n in zip(origin, gridsize, v.shape)]
    q = np.meshgrid(*[np.linspace(a[0], a[-1], n) for a, n in zip(axes, new_shape)],
                    indexing="ij")
    fn = RegularGridInterpolator(axes, v, method=method, bounds_error=False)
    return fn(np.stack([x.ravel() for x in q], axis=-1)).reshape(new_shape)


def test_reference_known_answers():
    eik = fp.Eikonal3D(np.ones((16, 16, 16)), (1.0, 1.0, 1.0))
    eik.resample((32, 32, 32))
    assert eik.grid.sum() == 16 * 16 * 16 * 8.0
    assert eik.gridsize == (0.5, 0.5, 0.5)
    eik = fp.Eikonal3D(np.ones((16, 16, 16)), (1.0, 1.0, 1.0))
    eik.smooth(1.0)
    assert np.isclose(eik.grid.sum(), eik.grid.size, rtol=1e-13)
    eik2 = fp.Eikonal2D(np.ones((16, 16)), (1.0, 1.0))
    eik2.resample((32, 32))
    assert eik2.grid.sum() == 16 * 16 * 4.0
    eik2 = fp.Eikonal2D(np.ones((16, 16)), (1.0, 1.0))
    eik2.smooth(1.0)
    assert np.isclose(eik2.grid.sum(), eik2.grid.size, rtol=1e-13)


@pytest.mark.parametrize("method", ["linear", "nearest"])
@pytest.mark.parametrize(
    "shape,new_shape,gridsize,origin",
    [((13, 17, 9), (30, 8, 21), (10.0, 7.0, 12.5), (5.0, -3.0, 100.0)),
     ((40, 33), (17, 95), (2.5, 4.0), (0.0, 10.0)),
     ((5, 6, 7), (5, 6, 7), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))],
)
def test_resample_matches_scipy(method, shape, new_shape, gridsize, origin):
    rng = np.random.default_rng(len(shape) * 10 + len(method))
    v = rng.uniform(1500.0, 4500.0, shape)
    ref = scipy_resample(v, gridsize, origin, new_shape, method)
    g = (fp.Eikonal3D if len(shape) == 3 else fp.Eikonal2D)(v, gridsize, origin)
    g.resample(new_shape, method)
    out = g.grid
    assert out.shape == ref.shape
    if method == "nearest":
        assert np.array_equal(out, ref)
    else:
        assert np.max(np.abs(out - ref) / np.abs(ref)) <= 1e-14
    assert np.allclose(g.gridsize, [a * b / c for a, b, c in zip(gridsize, shape, new_shape)],
                       rtol=0, atol=0)


@pytest.mark.parametrize(
    "shape,gridsize,sigma",
    [((20, 31, 17), (10.0, 10.0, 10.0), 25.0),
     ((12, 9, 40), (5.0, 8.0, 2.0), (10.0, 0.0, 30.0)),
     ((50, 64), (10.0, 4.0), 60.0),
     ((6, 7, 8), (1.0, 1.0, 1.0), 9.0)],  # kernel radius beyond the grid: repeated reflections
)
def test_smooth_matches_scipy(shape, gridsize, sigma):
    rng = np.random.default_rng(sum(shape))
    v = rng.uniform(1500.0, 4500.0, shape)
    sig = np.full(len(shape), sigma) if np.ndim(sigma) == 0 else np.asarray(sigma)
    ref = gaussian_filter(v, sig / np.asarray(gridsize))
    g = (fp.Eikonal3D if len(shape) == 3 else fp.Eikonal2D)(v, gridsize)
    g.smooth(sigma)
    assert np.max(np.abs(g.grid - ref) / np.abs(ref)) <= 1e-12


def test_prepared_model_solves_like_the_reference_pipeline():
    """resample + smooth, then solve: the traveltimes equal the oracle's solve
    of the SciPy-prepared model to 1e-12."""
    from oracle import oracle as O

    rng = np.random.default_rng(3)
    v = rng.uniform(2000.0, 3000.0, (10, 12, 14))
    d = (10.0, 10.0, 10.0)
    eik = fp.Eikonal3D(v, d)
    eik.resample((20, 24, 28))
    eik.smooth(15.0)
    ref = scipy_resample(v, d, (0.0, 0.0, 0.0), (20, 24, 28), "linear")
    h = tuple(a * b / c for a, b, c in zip(d, v.shape, (20, 24, 28)))
    ref = gaussian_filter(ref, 15.0 / np.asarray(h))
    tt = eik.solve([0.0, 50.0, 60.0]).grid
    tt_o = O.solve3d(1.0 / ref, h, [[0.0, 50.0, 60.0]], 2, False)[0][0]
    assert np.max(np.abs(tt - tt_o) / np.maximum(tt_o, 1e-300)) <= 1e-12
