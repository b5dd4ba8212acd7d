"""A 3D solve captured in a CUDA graph and replayed: fteik3d_solve_async
enqueues only capturable work (memsets, one copy of the sources from the
caller's pinned host buffer, kernel launches), so a loop that re-solves the
same problem (tomography iterations, new source positions) can replay it."""

import numpy as np
import pytest
import torch

from fteikpy_gb300 import _device, _lib
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_solve_replays_from_a_cuda_graph_with_new_sources():
    lib = _lib.load()
    rng = np.random.default_rng(12)
    shape, d = (18, 25, 22), (10.0, 10.0, 10.0)
    v = 2000.0 + 1000.0 * rng.uniform(0.0, 1.0, shape)
    slow = _device.slowness(_device.to_device(v))
    nz, nx, ny = shape
    nsrc = 6
    ext = np.array(shape) * np.array(d)
    src_a = rng.uniform(0.0, 1.0, (nsrc, 3)) * ext
    src_b = rng.uniform(0.0, 1.0, (nsrc, 3)) * ext
    pinned = torch.empty((nsrc, 3), dtype=torch.float64).pin_memory()
    dev = slow.device
    tt = torch.empty((nsrc, nz + 1, nx + 1, ny + 1), dtype=torch.float64, device=dev)
    tg = torch.empty((nsrc, nz + 1, nx + 1, ny + 1, 3), dtype=torch.float64, device=dev)
    vz = torch.empty(nsrc, dtype=torch.float64, device=dev)
    ws = torch.empty(lib.fteik3d_workspace_bytes(nz, nx, ny, nsrc, 1), dtype=torch.uint8,
                     device=dev)

    def enqueue(stream):
        return lib.fteik3d_solve_async(
            _device.ptr(slow), nz, nx, ny, *d, pinned.data_ptr(), nsrc, 2, 1, _device.ptr(tt),
            _device.ptr(tg), _device.ptr(vz), _device.ptr(ws), ws.numel(), 0, stream,
        )

    pinned.numpy()[:] = src_a
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):  # warm-up outside the capture
        assert enqueue(side.cuda_stream) == 0
    side.synchronize()
    assert lib.fteik_workspace_status(_device.ptr(ws), None) == 0
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        assert enqueue(torch.cuda.current_stream().cuda_stream) == 0
    for src in (src_a, src_b, src_a):
        pinned.numpy()[:] = src
        graph.replay()
        torch.cuda.synchronize()
        assert lib.fteik_workspace_status(_device.ptr(ws), None) == 0
        tt_o, tg_o, vz_o = O.solve3d(1.0 / v, d, src, 2, True)
        assert np.array_equal(tt.cpu().numpy(), tt_o)
        assert np.array_equal(tg.cpu().numpy(), tg_o)
        assert np.array_equal(vz.cpu().numpy(), vz_o)
