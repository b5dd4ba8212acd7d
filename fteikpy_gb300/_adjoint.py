"""Differentiable 3D traveltimes: receiver traveltimes as a function of the
velocity model, with a hand-written adjoint (``fteik3d_adjoint``).

The reference solver is not differentiable; this is the tomography extension
of the GPU path. The forward pass is the reference's solve
(``fteikpy/_fteik/_fteik3d.py``) followed by its apparent-velocity
interpolation at the receivers (``fteikpy/_interp/_vinterp3d.py``); the
backward pass maps d(loss)/d(receiver traveltimes) to d(loss)/d(velocity).
The forward solve keeps a tape of every sweep (``fteik3d_solve_tape``), and the
backward pass is the exact reverse-mode derivative of those sweeps, so it
matches finite differences of the solver for any ``nsweep``.
"""

import numpy as np
import torch

from . import _device, _lib
from ._solver import SPIN_LIMIT, solve3d_device


def _velocity(velocity):
    """The velocity model as a contiguous float64 tensor on the current CUDA
    device (converted when it is not one already), detached from autograd."""
    if not isinstance(velocity, torch.Tensor):
        raise TypeError("velocity must be a torch.Tensor [nz, nx, ny]")
    if velocity.dim() != 3:
        raise ValueError("velocity must have shape [nz, nx, ny]")
    return velocity.detach().to(device=_device.device(), dtype=torch.float64).contiguous()


def _points(points, what):
    """[n, 3] float64 host coordinates (a single point may be given as [3])."""
    p = np.ascontiguousarray(np.atleast_2d(np.asarray(points, dtype=np.float64)))
    if p.ndim != 2 or p.shape[-1] != 3 or len(p) == 0:
        raise ValueError(f"{what} must have shape (3,) or (n, 3)")
    return p


def _node_axes(shape, gridsize):
    return [_device.to_device(gridsize[d] * np.arange(shape[d] + 1)) for d in range(3)]


def _receiver_times(tt, axes, src_dev, vzero, receivers):
    """Traveltimes of every source at every receiver: [nsrc, nrec] (device)."""
    lib = _lib.load()
    nsrc = tt.shape[0]
    nrec = receivers.shape[0]
    pts = receivers.repeat(nsrc, 1).contiguous()
    gidx = torch.arange(nsrc, dtype=torch.int32, device=tt.device).repeat_interleave(nrec)
    out = torch.empty(nsrc * nrec, dtype=torch.float64, device=tt.device)
    rc = lib.fteik_vinterp3d(
        _device.ptr(axes[0]), len(axes[0]), _device.ptr(axes[1]), len(axes[1]),
        _device.ptr(axes[2]), len(axes[2]), _device.ptr(tt), tt[0].numel(), _device.ptr(gidx),
        _device.ptr(pts), nsrc * nrec, _device.ptr(src_dev), _device.ptr(vzero), float("nan"),
        _device.ptr(out), _device.stream(),
    )
    _lib.check(rc, "traveltimes")
    return out.view(nsrc, nrec)


class _Traveltimes(torch.autograd.Function):
    @staticmethod
    def forward(ctx, velocity, gridsize, sources, receivers, nsweep):
        lib = _lib.load()
        slow = _device.slowness(_velocity(velocity))
        ctx.velocity_meta = (velocity.dtype, velocity.device)
        nz, nx, ny = slow.shape
        src = _points(sources, "sources")
        receivers = _points(receivers, "receivers")
        nsrc = len(src)
        nsweep = max(int(nsweep), 0)
        dev = slow.device
        ws = torch.empty(lib.fteik3d_workspace_bytes(nz, nx, ny, nsrc, 2), dtype=torch.uint8,
                         device=dev)
        tape = torch.empty(lib.fteik3d_tape_bytes(nz, nx, ny, nsrc, nsweep), dtype=torch.uint8,
                           device=dev)
        tt = torch.empty((nsrc, nz + 1, nx + 1, ny + 1), dtype=torch.float64, device=dev)
        vzero = torch.empty(nsrc, dtype=torch.float64, device=dev)
        rc = lib.fteik3d_solve_tape(
            _device.ptr(slow), nz, nx, ny, *[float(g) for g in gridsize], _device.host_ptr(src),
            nsrc, nsweep, _device.ptr(tt), _device.ptr(vzero), _device.ptr(ws), ws.numel(),
            _device.ptr(tape), tape.numel(), SPIN_LIMIT, _device.stream(),
        )
        _lib.check(rc, "traveltimes")
        axes = _node_axes(slow.shape, gridsize)
        src_dev = _device.to_device(src)
        rec = _device.to_device(np.ascontiguousarray(receivers, dtype=np.float64))
        times = _receiver_times(tt, axes, src_dev, vzero, rec)
        ctx.save_for_backward(slow, tt, ws, tape, src_dev, rec)
        ctx.nsweep = nsweep
        ctx.gridsize = tuple(float(g) for g in gridsize)
        ctx.axes = axes
        return times

    @staticmethod
    def backward(ctx, grad_times):
        lib = _lib.load()
        slow, tt, ws, tape, src_dev, rec = ctx.saved_tensors
        nz, nx, ny = slow.shape
        nsrc = tt.shape[0]
        g = grad_times.detach().to(torch.float64).contiguous()
        grad_slow = torch.empty_like(slow)
        aws = torch.empty(
            lib.fteik3d_adjoint_workspace_bytes(nz, nx, ny, nsrc), dtype=torch.uint8,
            device=slow.device,
        )
        ax = ctx.axes
        rc = lib.fteik3d_adjoint(
            _device.ptr(slow), nz, nx, ny, *ctx.gridsize, nsrc, ctx.nsweep, _device.ptr(tt),
            _device.ptr(ws), ws.numel(), _device.ptr(tape), tape.numel(), _device.ptr(ax[0]),
            _device.ptr(ax[1]), _device.ptr(ax[2]),
            _device.ptr(src_dev), _device.ptr(rec), rec.shape[0], _device.ptr(g),
            _device.ptr(grad_slow), _device.ptr(aws), aws.numel(), SPIN_LIMIT, _device.stream(),
        )
        _lib.check(rc, "traveltimes backward")
        # slowness = 1 / velocity, so dL/dv = -dL/ds * s^2
        grad_velocity = -grad_slow * slow * slow
        dtype, device = ctx.velocity_meta
        return grad_velocity.to(device=device, dtype=dtype), None, None, None, None


def traveltimes(velocity, gridsize, sources, receivers, nsweep=2):
    """Traveltimes from every source to every receiver, differentiable in velocity.

    Parameters
    ----------
    velocity : torch.Tensor
        [nz, nx, ny] cell velocities (``requires_grad`` to get
        d(loss)/d(velocity)). The solve runs in float64 on the current CUDA
        device; a tensor of another dtype or device is converted, and its
        gradient comes back in its own dtype and device.
    gridsize : (dz, dx, dy)
    sources, receivers : array_like [n, 3] (or one point [3])
        Coordinates relative to the grid origin (node (0, 0, 0) at 0).
    nsweep : int
        Sweeps of the solve; the gradient is that of this many sweeps.

    Returns
    -------
    torch.Tensor [nsrc, nrec]: apparent-velocity interpolated traveltimes, the
    values ``TraveltimeGrid3D.__call__`` returns for an origin at 0.
    """
    return _Traveltimes.apply(velocity, tuple(gridsize), _points(sources, "sources"),
                              _points(receivers, "receivers"), int(nsweep))


def converged(velocity, gridsize, sources, nsweep):
    """True when one more sweep would leave every traveltime unchanged, i.e.
    when the derivative of ``traveltimes`` is the derivative of the solve."""
    slow = _device.slowness(_velocity(velocity))
    src = _points(sources, "sources")
    a, _, _ = solve3d_device(slow, gridsize, src, nsweep, False)
    a = a.clone()
    b, _, _ = solve3d_device(slow, gridsize, src, nsweep + 1, False)
    return bool(torch.equal(a, b))
