"""The 256-source batch at its full size (128 x 256 x 256 cells, 17.4 GB of
traveltimes, offsets past 2^31 elements): sampled sources equal their own
single-source solves (another kernel and schedule) and the oracle, bit for
bit."""

import os
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402
from fteikpy_gb300 import _device, _lib, _solver  # noqa: E402
from oracle import oracle as O  # noqa: E402


def test_full_size_batch_equals_single_solves_and_oracle():
    free, _ = torch.cuda.mem_get_info()
    if free < 24e9:
        pytest.skip("needs about 20 GB of free device memory")
    v = bench.layered_model()
    src = bench.surface_sources()
    assert len(src) == 256
    slow = _device.slowness(_device.to_device(v))
    tt, _, vz = _solver.solve3d_device(slow, bench.D, src, 2, False)
    assert _lib.load().fteik_last_sweep_kernel() == b"sweep3d_team_kernel"
    for s in (0, 97, 255):
        one, _, vz1 = _solver.solve3d_device(slow, bench.D, src[s:s + 1], 2, False)
        assert torch.equal(one[0].view(torch.int64), tt[s].view(torch.int64)), s
        assert float(vz1[0]) == float(vz[s])
    ref = O.solve3d(1.0 / v, bench.D, src[255:256], 2, False)[0][0]
    assert np.array_equal(tt[255].cpu().numpy(), ref)
