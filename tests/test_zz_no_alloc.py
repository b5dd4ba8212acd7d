"""The 3D solve that allocates nothing (fteik3d_solve_noalloc), through the C ABI.

Some callers cannot call cudaMalloc or hand the library a device workspace:
a framework that owns all device memory, a latency-critical loop where an
allocation would synchronise the device, a foreign-language binding that can
only pass the buffers it already owns. For them the library keeps the solver's
scratch in a fixed array of its own. This test checks that entry point against
the regular one (fteik3d_solve with a caller-provided workspace) on two calls in
a row, which share that array, and that a problem too large for the array is
refused before any GPU work.

The file name makes pytest collect it last; it also passes on its own in a
fresh process.
"""

import ctypes

import numpy as np
import pytest
import torch

from fteikpy_gb300 import _device, _lib

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the relative tolerance of the other parity tests


def _model(shape, seed):
    rng = np.random.default_rng(seed)
    v = np.linspace(1500.0, 3500.0, shape[0])[:, None, None] * np.ones(shape)
    return v * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, shape))


def _solve(lib, slow, d, src, nsweep, grad, noalloc, spin_limit=0, expect_ok=True):
    nz, nx, ny = slow.shape
    n = len(src)
    dev = slow.device
    tt = torch.empty((n, nz + 1, nx + 1, ny + 1), dtype=torch.float64, device=dev)
    tg = torch.empty((n, nz + 1, nx + 1, ny + 1, 3), dtype=torch.float64, device=dev) if grad else None
    vz = torch.empty(n, dtype=torch.float64, device=dev)
    srch = np.ascontiguousarray(src, dtype=np.float64)
    args = (_device.ptr(slow), nz, nx, ny, *d, srch.ctypes.data_as(ctypes.c_void_p), n, nsweep,
            int(grad), _device.ptr(tt), _device.ptr(tg), _device.ptr(vz))
    if noalloc:
        rc = lib.fteik3d_solve_noalloc(*args, spin_limit, _device.stream())
    else:
        ws = torch.empty(lib.fteik3d_workspace_bytes(nz, nx, ny, n, int(grad)), dtype=torch.uint8,
                         device=dev)
        rc = lib.fteik3d_solve(*args, _device.ptr(ws), ws.numel(), spin_limit, _device.stream())
    if not expect_ok:
        return rc
    assert rc == _lib.OK, (rc, lib.fteik_last_error())
    return tt.cpu().numpy(), (tg.cpu().numpy() if grad else None), vz.cpu().numpy()


def _rel(a, b):
    d = np.abs(a - b)
    return float(np.max(np.where(b != 0.0, d / np.where(b != 0.0, np.abs(b), 1.0), d)))


def test_noalloc_solve_matches_workspace_solve_twice():
    lib = _lib.load()
    torch.cuda.set_device(0)
    cases = [
        ((24, 30, 36), (10.0, 10.0, 10.0), np.array([[0.0, 123.4, 201.7], [55.5, 10.0, 300.0]]), 2, True, 1),
        ((17, 40, 21), (8.0, 12.0, 9.0), np.array([[3.0, 250.0, 100.0]]), 3, False, 2),
    ]
    for shape, d, src, nsweep, grad, seed in cases:  # two calls in a row share the scratch
        slow = _device.slowness(_device.to_device(_model(shape, seed)))
        a = _solve(lib, slow, d, src, nsweep, grad, noalloc=True)
        b = _solve(lib, slow, d, src, nsweep, grad, noalloc=False)
        assert _rel(a[0], b[0]) <= TOL
        assert np.array_equal(a[0], b[0])
        if grad:
            assert np.array_equal(a[1], b[1])
        assert np.array_equal(a[2], b[2])


def test_noalloc_team_kernel_after_a_timed_out_call():
    """The shared array after a call that gave up: a call whose device-side
    waits are limited to one poll (which may time out and leave a non-zero
    status and half-advanced counters in the array), then a regular call with
    blocks of several sources stepping together (6 sources, not a multiple of
    the block's 4), which must equal the workspace solve bit for bit."""
    lib = _lib.load()
    torch.cuda.set_device(0)
    shape, d = (20, 28, 36), (10.0, 10.0, 10.0)
    rng = np.random.default_rng(8)
    src = np.column_stack([rng.uniform(0, 200, 6), rng.uniform(0, 280, 6), rng.uniform(0, 360, 6)])
    slow = _device.slowness(_device.to_device(_model(shape, 4)))
    rc = _solve(lib, slow, d, src, 2, True, noalloc=True, spin_limit=1, expect_ok=False)
    assert rc in (_lib.OK, _lib.DEVICE_WAIT_TIMEOUT), (rc, lib.fteik_last_error())
    assert lib.fteik_set_option(b"sweep_team", 1) == _lib.OK
    try:
        for _ in range(2):
            a = _solve(lib, slow, d, src, 2, True, noalloc=True)
            assert lib.fteik_last_sweep_kernel() == b"sweep3d_team_kernel"
            b = _solve(lib, slow, d, src, 2, True, noalloc=False)
            assert _rel(a[0], b[0]) <= TOL
            assert np.array_equal(a[0], b[0])
            assert np.array_equal(a[1], b[1])
            assert np.array_equal(a[2], b[2])
    finally:
        lib.fteik_set_option(b"sweep_team", -1)


def test_noalloc_rejects_problems_above_the_fixed_scratch():
    lib = _lib.load()
    # 256 sources on a 128x256x256 grid with gradients need ~2.2 GB of scratch;
    # the check happens before any pointer is touched.
    fake = ctypes.c_void_p(0x1000)
    src = np.zeros((256, 3))
    rc = lib.fteik3d_solve_noalloc(fake, 128, 256, 256, 10.0, 10.0, 10.0,
                                   src.ctypes.data_as(ctypes.c_void_p), 256, 2, 1, fake, fake,
                                   fake, 0, None)
    assert rc == _lib.WORKSPACE_TOO_SMALL
    assert b"fixed maximum" in lib.fteik_last_error()
