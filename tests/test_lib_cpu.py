"""CPU-only checks of the CUDA library and the host-side logic (no GPU needed).

The library is built here (nvcc cross-compiles sm_103a), loaded with ctypes,
and must export every entry point that include/fteik_gb300.h declares. The
host-side validation of the C ABI (argument checks, source bounds, workspace
sizes) runs before any CUDA call, so it is exercised here through the C ABI
with placeholder pointers that are never dereferenced.
"""

import ctypes
import os
import re

import numpy as np
import pytest

import fteikpy_gb300 as fp
from fteikpy_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fteik_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fteik[0-9a-z_]*)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "fteik3d_solve" in names and "fteik2d_solve" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert set(declared_functions()) <= set(_lib.SIGNATURES)
    assert b"sm_103a" in lib.fteik_version()


def test_workspace_sizes(lib):
    small = lib.fteik3d_workspace_bytes(4, 5, 6, 1, 0)
    with_grad = lib.fteik3d_workspace_bytes(4, 5, 6, 1, 1)
    assert with_grad >= small + 5 * 6 * 7  # one branch-record byte per node
    assert lib.fteik3d_workspace_bytes(4, 5, 6, 8, 1) > with_grad
    assert lib.fteik3d_workspace_bytes(0, 5, 6, 1, 1) == 0
    assert lib.fteik2d_workspace_bytes(10, 12, 3, 1) >= 3 * 11 * 13
    for b in (small, with_grad, lib.fteik2d_workspace_bytes(10, 12, 3, 1)):
        assert b % 256 == 0


def test_tape_sizes_and_history_limits(lib):
    """The adjoint's tape: 8 * nsweep code bytes and 8 * history value bytes
    per node and source, plus the overflow table (a power of 2 of at least a
    quarter of the nodes, 16 bytes a slot) and per-source set-up; history is
    at most 8 * nsweep - 1 (0 without sweeps)."""
    nodes = 5 * 6 * 7
    n = nodes * 3
    cap = 4096
    while cap < n // 4:
        cap *= 2
    for nsweep, history in ((2, 2), (1, 7), (3, 0)):
        b = lib.fteik3d_tape_bytes(4, 5, 6, 3, nsweep, history)
        assert b % 256 == 0
        assert b >= n * (8 * nsweep + 8 * history) + 16 * cap + 3 * (64 + 48)
    big = 64 * 129 * 129 * 97
    assert lib.fteik3d_tape_bytes(96, 128, 128, 64, 2, 2) < 40 * big  # dense: 144 per node
    assert lib.fteik3d_tape_bytes(4, 5, 6, 3, 2, 16) == 0
    assert lib.fteik3d_tape_bytes(4, 5, 6, 3, 2, -1) == 0
    assert lib.fteik3d_tape_bytes(4, 5, 6, 3, 0, 0) > 0
    assert lib.fteik3d_tape_bytes(4, 5, 6, 3, 0, 1) == 0
    assert lib.fteik3d_tape_bytes(4, 5, 6, 3, 512, 2) == 0  # change numbers beyond 12 bits
    with pytest.raises(RuntimeError, match="tape overflowed"):
        _lib.check(_lib.TAPE_OVERFLOW)


def test_adjoint_chunk_plan():
    """The forward chunk (a taped solve) is the largest that fits beside the
    largest reverse-pass group that still fits; both halve down to one source."""
    from fteikpy_gb300 import _adjoint

    lib = _lib.load()
    k, g, need = _adjoint._chunk_plan(lib, (96, 128, 128), 64, 2, 1 << 50)
    assert (k, g) == (64, 64)
    # the reverse pass splits first: the solve of all 64 sources stays whole
    k2, g2, need2 = _adjoint._chunk_plan(lib, (96, 128, 128), 64, 2, need // 3)
    assert k2 == 64 and g2 < 64 and need2 <= need // 3
    k3, g3, need3 = _adjoint._chunk_plan(lib, (96, 128, 128), 64, 2, need // 8)
    assert k3 < 64 and g3 <= k3 and need3 <= need // 8
    assert _adjoint._chunk_plan(lib, (96, 128, 128), 64, 2, 1)[:2] == (1, 1)
    # 128x256x256, 64 sources under 40 GB: one solve, reverse pass in groups
    k4, g4, need4 = _adjoint._chunk_plan(lib, (128, 256, 256), 64, 2, 40 * 10**9)
    assert k4 == 64 and g4 < 64 and need4 <= 40 * 10**9
    assert _adjoint._history_steps(2) == [2, 6, 15]
    assert _adjoint._history_steps(1) == [2, 6, 7]
    assert _adjoint._history_steps(0) == [0]


FAKE = ctypes.c_void_p(0x1000)  # never dereferenced: the calls fail host-side first


def _solve3d(lib, src, nz=4, nx=5, ny=6, d=(1.0, 1.0, 1.0), ws_bytes=None, nsweep=2):
    src = np.ascontiguousarray(np.atleast_2d(src), dtype=np.float64)
    ws = ws_bytes if ws_bytes is not None else lib.fteik3d_workspace_bytes(nz, nx, ny, len(src), 1)
    return lib.fteik3d_solve(
        FAKE, nz, nx, ny, *d, src.ctypes.data_as(ctypes.c_void_p), len(src), nsweep, 1, FAKE,
        FAKE, FAKE, FAKE, ws, 0, None,
    )


def test_models_above_2_31_nodes_are_refused_host_side(lib):
    """The sweep kernels index a model's nodes with 32-bit integers: a model
    of 2^31 nodes or more is refused before any device work, with a message."""
    src = np.zeros((1, 3))
    rc = lib.fteik3d_solve(FAKE, 1290, 1290, 1290, 1.0, 1.0, 1.0,
                           src.ctypes.data_as(ctypes.c_void_p), 1, 2, 0, FAKE, FAKE, FAKE, FAKE,
                           1 << 62, 0, None)
    assert rc == _lib.INVALID_ARGUMENT
    assert b"2^31" in lib.fteik_last_error()


def test_source_out_of_bound_is_host_side(lib):
    # fteikpy/_fteik/_fteik3d.py:403-407: 0 <= src <= d * n on every axis
    assert _solve3d(lib, [4.0 + 1e-9, 0.0, 0.0]) == _lib.SOURCE_OUT_OF_BOUND
    assert _solve3d(lib, [0.0, -1e-12, 0.0]) == _lib.SOURCE_OUT_OF_BOUND
    assert _solve3d(lib, [[1.0, 1.0, 1.0], [0.0, 0.0, 6.5]]) == _lib.SOURCE_OUT_OF_BOUND
    assert _solve3d(lib, [np.nan, 0.0, 0.0]) == _lib.SOURCE_OUT_OF_BOUND
    src = np.ascontiguousarray([[0.0, 5.5, 0.0]])
    rc = lib.fteik2d_solve(FAKE, 4, 5, 1.0, 1.0, src.ctypes.data_as(ctypes.c_void_p), 1, 2, 1,
                           FAKE, FAKE, FAKE, FAKE, lib.fteik2d_workspace_bytes(4, 5, 1, 1), None)
    assert rc == _lib.SOURCE_OUT_OF_BOUND


def test_invalid_arguments_are_host_side(lib):
    assert _solve3d(lib, [0.0, 0.0, 0.0], ws_bytes=16) == _lib.WORKSPACE_TOO_SMALL
    assert _solve3d(lib, [0.0, 0.0, 0.0], nz=1) == _lib.INVALID_ARGUMENT
    assert _solve3d(lib, [0.0, 0.0, 0.0], d=(0.0, 1.0, 1.0)) == _lib.INVALID_ARGUMENT
    assert _solve3d(lib, [0.0, 0.0, 0.0], nsweep=-1) == _lib.INVALID_ARGUMENT
    rc = lib.fteik3d_solve(None, 4, 5, 6, 1.0, 1.0, 1.0, None, 1, 2, 0, None, None, None, None,
                           0, 0, None)
    assert rc == _lib.INVALID_ARGUMENT
    assert lib.fteik_ray_pack(4, FAKE, 1, 10, FAKE, FAKE, FAKE, None) == _lib.INVALID_ARGUMENT
    assert lib.fteik_ray3d(FAKE, 3, FAKE, 3, FAKE, 3, FAKE, 0, None, FAKE, 1, FAKE, 1.0, 1, 0,
                           FAKE, FAKE, FAKE, None) == _lib.INVALID_ARGUMENT


def test_status_codes_map_to_reference_exceptions():
    with pytest.raises(ValueError, match="source out of bound"):
        _lib.check(_lib.SOURCE_OUT_OF_BOUND)
    with pytest.raises(ValueError, match="end point out of bound"):
        _lib.check(_lib.END_POINT_OUT_OF_BOUND)
    with pytest.raises(RuntimeError, match="maximum number of steps reached"):
        _lib.check(_lib.MAX_STEP_REACHED)
    with pytest.raises(RuntimeError, match="timed out"):
        _lib.check(_lib.DEVICE_WAIT_TIMEOUT)
    _lib.check(_lib.OK)


def test_api_host_logic():
    # fteikpy tests/test_misc.py:4-7
    fp.set_num_threads(1)
    assert fp.get_num_threads() == 1
    v = np.full((4, 5, 6), 2.0)
    eik = fp.Eikonal3D(v, (1.0, 2.0, 3.0), origin=(1.0, 0.0, -1.0))
    assert eik.shape == (4, 5, 6) and eik.ndim == 3 and eik.size == 120
    assert eik.gridsize == (1.0, 2.0, 3.0)
    assert np.array_equal(eik.zaxis, 1.0 + np.arange(4))
    assert np.array_equal(eik.yaxis, -1.0 + 3.0 * np.arange(6))
    assert eik[0, 0, 0] == 2.0
    tt = fp.TraveltimeGrid3D(np.zeros((5, 6, 7)), (1.0, 1.0, 1.0), np.zeros(3), [0, 0, 0], None, 1.0)
    with pytest.raises(ValueError, match="no gradient grid"):
        tt.gradient
    with pytest.raises(ValueError, match="no gradient grid"):
        tt.raytrace([1.0, 1.0, 1.0])
    tt2 = fp.TraveltimeGrid2D(np.zeros((5, 6)), (1.0, 1.0), np.zeros(2), [0, 0], None, 1.0)
    with pytest.raises(ValueError, match="no gradient grid"):
        tt2.gradient
    with pytest.raises(ValueError, match="no gradient grid"):
        tt2.gradient_tensor


def test_traveltimes_argument_checks_are_host_side():
    """The differentiable traveltimes reject what the kernels could misread
    before any device call: a velocity that is not a 3D tensor, and point
    lists that are not [n, 3] (one point may be given as [3])."""
    import torch

    from fteikpy_gb300 import _adjoint

    with pytest.raises(TypeError):
        fp.traveltimes(np.ones((4, 5, 6)), (1.0, 1.0, 1.0), [[0, 1, 1]], [[0, 2, 2]])
    with pytest.raises(ValueError, match="velocity must have shape"):
        _adjoint._velocity(torch.ones((4, 5)))
    with pytest.raises(ValueError, match="receivers must have shape"):
        _adjoint._points([0.0, 1.0], "receivers")
    with pytest.raises(ValueError, match="sources must have shape"):
        _adjoint._points(np.zeros((2, 2)), "sources")
    assert _adjoint._points([0.0, 1.0, 2.0], "receivers").shape == (1, 3)


def test_grid_ops_host_checks(lib):
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    d3 = np.ascontiguousarray([4, 5, 6], dtype=np.int32)
    bad = np.ascontiguousarray([4, 0, 6], dtype=np.int32)
    one = np.ascontiguousarray([1, 5, 6], dtype=np.int32)
    INV = _lib.INVALID_ARGUMENT
    # no GPU needed: every call below fails its host-side checks first
    assert lib.fteik_resample(0, 0, FAKE, p(d3), p(d3), FAKE, FAKE, FAKE, FAKE, None) == INV
    assert lib.fteik_resample(3, 0, FAKE, p(bad), p(d3), FAKE, FAKE, FAKE, FAKE, None) == INV
    assert lib.fteik_resample(3, 0, FAKE, p(one), p(d3), FAKE, FAKE, FAKE, FAKE, None) == INV
    assert lib.fteik_resample(3, 0, FAKE, p(d3), p(d3), FAKE, None, FAKE, FAKE, None) == INV
    w = ctypes.c_void_p(0x2000)
    assert lib.fteik_correlate1d(3, FAKE, p(d3), 3, w, 5, w, None) == INV
    assert lib.fteik_correlate1d(3, FAKE, p(d3), 0, w, 4, w, None) == INV
    assert lib.fteik_correlate1d(3, FAKE, p(d3), 0, w, 5, FAKE, None) == INV  # in place


def test_grid_op_tables_follow_scipy():
    """The host half of resample/smooth: per-axis lookups and Gaussian
    weights, checked against SciPy (the device half runs in the GPU tests)."""
    from scipy.interpolate import RegularGridInterpolator
    from scipy.ndimage import gaussian_filter1d

    from fteikpy_gb300._base import _axis_table, _gaussian_weights

    axis = 3.0 + 7.5 * np.arange(11)
    q = np.linspace(axis[0], axis[-1], 29)
    i, y, ym = _axis_table(axis, q, "linear")
    vals = np.random.default_rng(0).uniform(1, 2, 11)
    lin = vals[i] * ym + vals[i + 1] * y
    ref = RegularGridInterpolator((axis,), vals)(q[:, None])
    assert np.allclose(lin, ref, rtol=1e-15, atol=0)
    near, _, _ = _axis_table(axis, q, "nearest")
    ref = RegularGridInterpolator((axis,), vals, method="nearest")(q[:, None])
    assert np.array_equal(vals[near], ref)
    for sigma in (0.3, 1.0, 2.7):
        w = _gaussian_weights(sigma)
        x = np.zeros(4 * len(w) + 1)
        x[len(x) // 2] = 1.0
        assert np.allclose(gaussian_filter1d(x, sigma)[len(x) // 2 - len(w) // 2:][:len(w)],
                           w[::-1], rtol=1e-14, atol=1e-17)


def _batch_args(dims, nsrc, sources, spacing=None):
    n = len(dims)
    P = ctypes.c_void_p * n
    dims = np.ascontiguousarray(dims, dtype=np.int32)
    nsrc = np.ascontiguousarray(nsrc, dtype=np.int32)
    spacing = np.ascontiguousarray(spacing if spacing is not None else np.ones((n, 3)))
    sources = np.ascontiguousarray(sources, dtype=np.float64)
    return n, P(*[FAKE] * n), dims, spacing, sources, nsrc, P(*[FAKE] * n)


def test_batch_workspace_and_host_checks(lib):
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    dims = [[4, 5, 6], [9, 3, 7]]
    d = np.ascontiguousarray(dims, dtype=np.int32)
    one = np.ascontiguousarray([1, 1], dtype=np.int32)
    two = np.ascontiguousarray([20, 30], dtype=np.int32)
    b1 = lib.fteik3d_batch_workspace_bytes(2, p(d), p(one), 0)
    assert b1 > 0 and b1 % 256 == 0
    assert lib.fteik3d_batch_workspace_bytes(2, p(d), p(two), 0) > b1
    assert lib.fteik3d_batch_workspace_bytes(2, p(d), p(two), 1) > lib.fteik3d_batch_workspace_bytes(
        2, p(d), p(two), 0)
    bad = np.ascontiguousarray([[4, 5, 6], [0, 3, 7]], dtype=np.int32)
    assert lib.fteik3d_batch_workspace_bytes(2, p(bad), p(one), 0) == 0
    assert lib.fteik3d_batch_workspace_bytes(0, p(d), p(one), 0) == 0

    def solve(sources, nsrc=(1, 1), grad=0, ws=None, dims=dims):
        n, slow, dd, sp, src, ns, tt = _batch_args(dims, nsrc, sources)
        wsb = ws if ws is not None else lib.fteik3d_batch_workspace_bytes(n, p(dd), p(ns), grad)
        return lib.fteik3d_solve_batch(n, slow, p(dd), p(sp), p(src), p(ns), 2, grad, tt,
                                       tt if grad else None, FAKE, FAKE, wsb, 0, None)

    # model 1 is 9 x 3 x 7 cells of 1 m: z = 9.5 is outside
    assert solve([[0.0, 0.0, 0.0], [9.5, 0.0, 0.0]]) == _lib.SOURCE_OUT_OF_BOUND
    assert solve([[4.5, 0.0, 0.0], [0.0, 0.0, 0.0]]) == _lib.SOURCE_OUT_OF_BOUND
    assert solve([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]], ws=256) == _lib.WORKSPACE_TOO_SMALL
    assert solve([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]], grad=2) == _lib.INVALID_ARGUMENT
    assert solve([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]],
                 dims=[[4, 5, 6], [1, 3, 7]]) == _lib.INVALID_ARGUMENT


def test_tuning_options_host_side(lib):
    v = ctypes.c_longlong()
    for name, good, bad in ((b"sweep_pencil", (2, 4, 8), (1, 3, 16)),
                            (b"sweep_chunk", (1, 2, 64), (3, 0, 128)),
                            (b"sweep_coef", (0, 1), ()),
                            (b"sweep_keep_test", (0, 1), ()),
                            (b"sweep_team", (0, 1), ()),
                            (b"adjoint_chunk", (1, 4, 64), (3, 0, 128)),
                            (b"sweep2d_keys", (0, 1), ()),
                            (b"sweep2d_warp", (0, 1, 2), (3,)),
                            (b"sweep2d_speculate", (0, 1), ()),
                            (b"sweep2d_wait_ns", (0, 1000, 10**10), ()),
                            (b"ray_lanes", (1, 4, 32), (0, 2, 8, 64))):
        for g in good:
            assert lib.fteik_set_option(name, g) == 0
            assert lib.fteik_get_option(name, ctypes.byref(v)) == 0 and v.value == g
        for b in bad:
            assert lib.fteik_set_option(name, b) == _lib.INVALID_ARGUMENT
        assert lib.fteik_set_option(name, -1) == 0
    assert lib.fteik_set_option(b"no_such_option", 1) == _lib.INVALID_ARGUMENT
    assert lib.fteik_clear_tuning() == 0
