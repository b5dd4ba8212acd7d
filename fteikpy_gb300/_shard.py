"""Sources split across GPUs: the reference's parallel loop over sources
(``fteikpy/_fteik/_fteik3d.py:508``, numba ``prange``) across devices or ranks.

Sources are independent solves on one shared velocity model, so a source list
splits into contiguous shards, one per device (or per process of a
``torch.distributed`` group), with the model replicated; nothing is exchanged
during the solve. The one reduction is the adjoint's: d(loss)/d(velocity) is a
sum over sources, so the ranks' gradients are gathered and summed in rank
order (the same bits on every rank, whatever the collective's internal
order).
"""

import threading

import numpy as np
import torch

from . import _adjoint


def shard_bounds(n, parts, index):
    """[lo, hi) of shard ``index`` of ``parts`` contiguous, balanced shards of
    ``n`` items (the first n % parts shards hold one more)."""
    if parts < 1 or not 0 <= index < parts:
        raise ValueError("need 0 <= index < parts")
    base, extra = divmod(int(n), int(parts))
    lo = index * base + min(index, extra)
    return lo, lo + base + (1 if index < extra else 0)


def _solve_on(device, solver, sources, nsweep, return_gradient):
    """One shard's solve on ``device``: a copy of the solver whose model lives
    there, returning what ``Eikonal3D.solve`` returns for a list of sources."""
    with torch.cuda.device(device):
        eik = type(solver)(solver._device_grid().to(device), solver.gridsize, solver.origin)
        return eik.solve(sources, nsweep=nsweep, return_gradient=return_gradient)


def solve_sharded(solver, sources, nsweep=2, return_gradient=False, devices=None):
    """``solver.solve(sources, ...)`` for a list of sources, split across CUDA
    devices: device k solves the k-th contiguous shard, all at once (one host
    thread per device; the solves release the GIL). Returns the results in
    source order, each living on the device that solved it. No counterpart in
    the reference, whose numba ``prange`` spreads sources over CPU threads.

    ``devices``: CUDA device indices (default: every visible device).
    """
    src = np.atleast_2d(np.asarray(sources, dtype=np.float64))
    if devices is None:
        devices = list(range(torch.cuda.device_count()))
    devices = [int(d) for d in devices]
    if not devices:
        raise RuntimeError("solve_sharded needs at least one CUDA device")
    if len(set(devices)) != len(devices):
        # a device's solves share its scratch workspace: one shard per device
        raise ValueError("solve_sharded takes each device at most once")
    parts = min(len(devices), len(src))
    results = [None] * parts
    errors = [None] * parts

    def work(k):
        lo, hi = shard_bounds(len(src), parts, k)
        try:
            results[k] = _solve_on(devices[k], solver, src[lo:hi], nsweep, return_gradient)
        except Exception as e:  # re-raised in the caller's thread
            errors[k] = e

    threads = [threading.Thread(target=work, args=(k,)) for k in range(1, parts)]
    for t in threads:
        t.start()
    work(0)
    for t in threads:
        t.join()
    for e in errors:
        if e is not None:
            raise e
    out = []
    for r in results:
        out.extend(r)
    return out


def sum_in_rank_order(t, group=None):
    """Sum of ``t`` over the ranks of ``group``, added in rank order on every
    rank (all-gather, then a sequential sum), so that all ranks hold the same
    bits and a rerun gives them again."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t.contiguous(), group=group)
    out = parts[0].clone()
    for p in parts[1:]:
        out += p
    return out


class _SumGradOverRanks(torch.autograd.Function):
    """Identity forward; the backward sums the gradient over the group's ranks
    in rank order."""

    @staticmethod
    def forward(ctx, velocity, group):
        ctx.group = group
        return velocity.view_as(velocity)

    @staticmethod
    def backward(ctx, grad):
        return sum_in_rank_order(grad, ctx.group), None


def _local_traveltimes(velocity, gridsize, sources, receivers, nsweep, memory_budget):
    return _adjoint.traveltimes(velocity, gridsize, sources, receivers, nsweep, memory_budget)


def sharded_traveltimes(velocity, gridsize, sources, receivers, nsweep=2, group=None,
                        memory_budget=None):
    """``traveltimes`` with the sources split across the ranks of a
    ``torch.distributed`` group (one process per GPU): this rank solves its
    contiguous shard (``shard_bounds``) and returns its [n_local, nrec]
    receiver traveltimes; the backward pass gives every rank the same
    d(loss)/d(velocity), the sum over all ranks' losses, added in rank order.

    Returns (traveltimes of this rank's sources, (lo, hi) of its shard)."""
    import torch.distributed as dist

    src = np.atleast_2d(np.asarray(sources, dtype=np.float64))
    world = dist.get_world_size(group)
    if len(src) < world:
        # every rank must run the backward pass's collective
        raise ValueError("sharded_traveltimes needs at least one source per rank")
    lo, hi = shard_bounds(len(src), world, dist.get_rank(group))
    v = _SumGradOverRanks.apply(velocity, group)
    return _local_traveltimes(v, gridsize, src[lo:hi], receivers, nsweep, memory_budget), (lo, hi)
