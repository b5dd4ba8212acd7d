"""Device plumbing: CUDA tensors, the current stream and scratch workspaces.

PyTorch provides device memory and streams; all computation happens in the
library's own kernels (``fteikpy_gb300/_lib.py``).
"""

import ctypes

import numpy as np
import torch

from . import _lib


def device():
    if not torch.cuda.is_available():
        raise RuntimeError(
            "fteikpy_gb300 runs on a CUDA GPU (GB300, sm_103a) and has no CPU fallback: "
            "no CUDA device is available"
        )
    return torch.device("cuda", torch.cuda.current_device())


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def host_ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def to_device(a, dtype=torch.float64):
    """Contiguous device tensor holding ``a`` (a NumPy array, a sequence or a tensor)."""
    if isinstance(a, torch.Tensor):
        return a.to(device=device(), dtype=dtype).contiguous()
    arr = np.ascontiguousarray(a, dtype=np.float64 if dtype == torch.float64 else None)
    return torch.from_numpy(arr).to(device=device(), dtype=dtype)


class Workspace:
    """A growable scratch buffer handed to the C ABI (which never allocates)."""

    def __init__(self):
        self._buf = None

    def get(self, nbytes):
        nbytes = max(int(nbytes), 256)
        if self._buf is None or self._buf.numel() < nbytes or self._buf.device != device():
            self._buf = torch.empty(nbytes, dtype=torch.uint8, device=device())
        return self._buf


_workspaces = {}


def workspace(key, nbytes):
    """The growable scratch buffer ``key`` of the current device (one per
    device, so that solves on several devices at once keep their own)."""
    ws = _workspaces.setdefault((key, device().index), Workspace())
    return ws.get(nbytes)


def slowness(velocity):
    """Device slowness 1 / velocity computed by the library (fteikpy/_solver.py:49,121)."""
    lib = _lib.load()
    v = velocity if velocity.is_contiguous() else velocity.contiguous()
    out = torch.empty_like(v)
    flag = workspace("slowness-flag", 256)
    rc = lib.fteik_slowness(ptr(v), v.numel(), ptr(out), ptr(flag), stream())
    if rc == _lib.INVALID_ARGUMENT:
        raise ValueError(
            "velocity model must hold finite values whose inverse lies in (1e-150, 1e150)"
        )
    _lib.check(rc, "slowness")
    return out
