"""Differentiable 3D traveltimes: receiver traveltimes as a function of the
velocity model, with a hand-written adjoint (``fteik3d_adjoint``).

The reference solver is not differentiable; this is the tomography extension
of the GPU path. The forward pass is the reference's solve
(``fteikpy/_fteik/_fteik3d.py``) followed by its apparent-velocity
interpolation at the receivers (``fteikpy/_interp/_vinterp3d.py``); the
backward pass maps d(loss)/d(receiver traveltimes) to d(loss)/d(velocity).
The forward solve keeps a tape of every change its sweeps make
(``fteik3d_solve_tape``), and the backward pass is the exact reverse-mode
derivative of those sweeps, so it matches finite differences of the solver for
any ``nsweep``. Sources run in chunks sized to a device-memory budget, and the
backward pass in groups of sources; a chunk whose tape is not kept is solved
again in the backward pass.
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


# History slots of the tape per node: the values replaced by a node's 2nd and
# 3rd changes (its later changes go to the tape's overflow table). A solve
# whose table overflows is run again with more slots.
HISTORY = 2
# Share of the free device memory one differentiable solve may take for its
# tapes and workspaces when no budget is given.
BUDGET_SHARE = 0.8


def _history_steps(nsweep):
    """The history slot counts to try in turn: 2, 6, then every sweep's."""
    top = max(8 * nsweep - 1, 0)
    steps = [h for h in (HISTORY, 6) if h < top]
    return steps + [top]


def _taped_solve(lib, slow, gridsize, src, nsweep, history, workspace):
    """fteik3d_solve_tape for the sources ``src`` (host [k, 3]); retries with
    more history slots while the tape's overflow table is too small. Returns
    (tt, vzero, tape, history)."""
    nz, nx, ny = slow.shape
    k = len(src)
    dev = slow.device
    tt = torch.empty((k, nz + 1, nx + 1, ny + 1), dtype=torch.float64, device=dev)
    vzero = torch.empty(k, dtype=torch.float64, device=dev)
    steps = [history] if history is not None else _history_steps(nsweep)
    for h in steps:
        tape = torch.empty(lib.fteik3d_tape_bytes(nz, nx, ny, k, nsweep, h), dtype=torch.uint8,
                           device=dev)
        rc = lib.fteik3d_solve_tape(
            _device.ptr(slow), nz, nx, ny, *gridsize, _device.host_ptr(src), k, nsweep,
            _device.ptr(tt), _device.ptr(vzero), _device.ptr(workspace), workspace.numel(), h,
            _device.ptr(tape), tape.numel(), SPIN_LIMIT, _device.stream(),
        )
        if rc != _lib.TAPE_OVERFLOW:
            _lib.check(rc, "traveltimes")
            return tt, vzero, tape, h
        del tape
    _lib.check(rc, "traveltimes")


def _halvings(n):
    """n, then n halved (rounded up) down to 1."""
    out = [n]
    while out[-1] > 1:
        out.append((out[-1] + 1) // 2)
    return out


def _chunk_plan(lib, shape, nsrc, nsweep, budget):
    """(k, group, need): sources per forward chunk (one taped solve), sources
    per group of the reverse pass, and the bytes a chunk's solve plus a
    group's reverse pass take.

    The forward chunk holds traveltimes, the tape and the solve's workspace
    (about 48 bytes per node and source); the reverse pass needs 136 more per
    node and source of its group, but runs group by group over a kept tape
    (fteik3d_adjoint_part). So the largest chunk is taken whose solve fits
    beside the largest group that still fits (at least one source each):
    fewer, larger solves run faster, and the groups only split the reverse
    pass, whose result does not depend on them."""
    nz, nx, ny = shape
    nodes = (nz + 1) * (nx + 1) * (ny + 1)
    hist = min(HISTORY, max(8 * nsweep - 1, 0))
    for k in _halvings(nsrc):
        solve = (8 * nodes * k + lib.fteik3d_workspace_bytes(nz, nx, ny, k, 2)
                 + lib.fteik3d_tape_bytes(nz, nx, ny, k, nsweep, hist))
        for g in _halvings(k):
            need = solve + lib.fteik3d_adjoint_workspace_bytes(nz, nx, ny, g)
            if need <= budget:
                return k, g, need
    return 1, 1, need


class _Traveltimes(torch.autograd.Function):
    @staticmethod
    def forward(ctx, velocity, gridsize, sources, receivers, nsweep, budget):
        lib = _lib.load()
        slow = _device.slowness(_velocity(velocity))
        ctx.velocity_meta = (velocity.dtype, velocity.device)
        nz, nx, ny = slow.shape
        src = _points(sources, "sources")
        receivers = _points(receivers, "receivers")
        nsrc = len(src)
        nsweep = max(int(nsweep), 0)
        gs = tuple(float(g) for g in gridsize)
        dev = slow.device
        if budget is None:
            budget = int(BUDGET_SHARE * torch.cuda.mem_get_info(dev)[0])
        k, group, chunk_bytes = _chunk_plan(lib, slow.shape, nsrc, nsweep, int(budget))
        group_bytes = lib.fteik3d_adjoint_workspace_bytes(nz, nx, ny, group)
        axes = _node_axes(slow.shape, gs)
        src_dev = _device.to_device(src)
        rec = _device.to_device(receivers)
        times = torch.empty((nsrc, len(receivers)), dtype=torch.float64, device=dev)
        ws = torch.empty(lib.fteik3d_workspace_bytes(nz, nx, ny, k, 2), dtype=torch.uint8,
                         device=dev)
        # Keep the chunks' traveltimes and tapes for the backward pass, from the
        # first chunk on, while they fit beside the next chunk's solve and one
        # group's reverse pass; once one is dropped, the later ones are too
        # (the backward pass solves them again, after the kept ones are freed).
        kept_bytes, keeping, chunks = 0, True, []
        solve_bytes = chunk_bytes - group_bytes
        for a in range(0, nsrc, k):
            b = min(a + k, nsrc)
            tt, vzero, tape, h = _taped_solve(lib, slow, gs, src[a:b], nsweep, None, ws)
            times[a:b] = _receiver_times(tt, axes, src_dev[a:b], vzero, rec)
            size = tt.numel() * 8 + tape.numel()
            after = kept_bytes + size
            keeping = keeping and after + group_bytes <= budget and (
                b == nsrc or after + solve_bytes <= budget)
            if keeping:
                kept_bytes = after
                chunks.append((a, b, h, tt, tape))
            else:
                chunks.append((a, b, h, None, None))
            del tt, tape
        ctx.save_for_backward(slow, src_dev, rec)
        ctx.src = src
        ctx.chunks = chunks
        ctx.group = group
        ctx.nsweep = nsweep
        ctx.gridsize = gs
        ctx.axes = axes
        return times

    @staticmethod
    def backward(ctx, grad_times):
        lib = _lib.load()
        slow, src_dev, rec = ctx.saved_tensors
        nz, nx, ny = slow.shape
        g = grad_times.detach().to(torch.float64).contiguous()
        grad_slow = torch.empty_like(slow)
        ax = ctx.axes
        ws = None
        aws = torch.empty(lib.fteik3d_adjoint_workspace_bytes(nz, nx, ny, ctx.group),
                          dtype=torch.uint8, device=slow.device)
        first = True
        for c, (a, b, h, tt, tape) in enumerate(ctx.chunks):
            ctx.chunks[c] = None  # freed once this chunk is done
            k = b - a
            if tt is None:  # not kept: solve this chunk again (same tape, same bits)
                if ws is None:
                    ws = torch.empty(lib.fteik3d_workspace_bytes(nz, nx, ny, k, 2),
                                     dtype=torch.uint8, device=slow.device)
                tt, _, tape, _ = _taped_solve(lib, slow, ctx.gridsize, ctx.src[a:b], ctx.nsweep,
                                              h, ws)
            # the reverse pass in groups of sources, the gradient summed on in
            # source order
            for g0 in range(0, k, ctx.group):
                n = min(ctx.group, k - g0)
                rc = lib.fteik3d_adjoint_part(
                    _device.ptr(slow), nz, nx, ny, *ctx.gridsize, k, g0, n, ctx.nsweep,
                    _device.ptr(tt), h, _device.ptr(tape), tape.numel(), _device.ptr(ax[0]),
                    _device.ptr(ax[1]), _device.ptr(ax[2]), _device.ptr(src_dev[a:b]),
                    _device.ptr(rec), rec.shape[0], _device.ptr(g[a:b]), int(not first),
                    _device.ptr(grad_slow), _device.ptr(aws), aws.numel(), SPIN_LIMIT,
                    _device.stream(),
                )
                _lib.check(rc, "traveltimes backward")
                first = False
            del tt, tape
        ctx.chunks = None
        # slowness = 1 / velocity, so dL/dv = -dL/ds * s^2
        grad_velocity = -grad_slow * slow * slow
        dtype, device = ctx.velocity_meta
        return grad_velocity.to(device=device, dtype=dtype), None, None, None, None, None


def traveltimes(velocity, gridsize, sources, receivers, nsweep=2, memory_budget=None):
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
    memory_budget : int or None
        Device bytes the solve's tapes and workspaces may take (default: 80%
        of the free device memory). The reverse pass runs in groups of
        sources over each solve's tape, and sources are solved in consecutive
        chunks when one solve of all of them does not fit; the tapes of the
        chunks that do not fit beside the others are dropped after the
        forward pass and solved again in the backward pass. The gradient's
        bits do not depend on the chunking or the grouping.

    Returns
    -------
    torch.Tensor [nsrc, nrec]: apparent-velocity interpolated traveltimes, the
    values ``TraveltimeGrid3D.__call__`` returns for an origin at 0.
    """
    return _Traveltimes.apply(velocity, tuple(gridsize), _points(sources, "sources"),
                              _points(receivers, "receivers"), int(nsweep), memory_budget)


def converged(velocity, gridsize, sources, nsweep):
    """True when one more sweep would leave every traveltime unchanged, i.e.
    when the derivative of ``traveltimes`` is the derivative of the solve."""
    slow = _device.slowness(_velocity(velocity))
    src = _points(sources, "sources")
    a, _, _ = solve3d_device(slow, gridsize, src, nsweep, False)
    a = a.clone()
    b, _, _ = solve3d_device(slow, gridsize, src, nsweep + 1, False)
    return bool(torch.equal(a, b))
