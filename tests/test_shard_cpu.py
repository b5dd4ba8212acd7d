"""Sources split across GPUs (``fteikpy_gb300._shard``), host logic on CPU.

The device solve is replaced by stand-ins that run on the CPU, so the
partition of a source list, the merge of the shards' results in source order,
and the adjoint's reduction over ranks (all-gather, then a sum in rank order,
the same bits on every rank) are checked with gloo ranks (world size 2) and
no GPU.
"""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from fteikpy_gb300 import _shard


def test_shard_bounds_cover_the_list_in_order():
    for n in (0, 1, 5, 7, 256, 1001):
        for parts in (1, 2, 3, 8):
            b = [_shard.shard_bounds(n, parts, k) for k in range(parts)]
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[k][1] == b[k + 1][0] for k in range(parts - 1))
            sizes = [hi - lo for lo, hi in b]
            assert max(sizes) - min(sizes) <= 1 and sorted(sizes, reverse=True) == sizes
    with pytest.raises(ValueError):
        _shard.shard_bounds(10, 2, 2)


def test_solve_sharded_merges_shards_in_source_order(monkeypatch):
    """Device k gets the k-th contiguous shard; the results come back in
    source order whatever order the threads finish in."""
    import threading
    import time

    seen = {}
    lock = threading.Lock()

    def fake_solve_on(device, solver, sources, nsweep, return_gradient):
        time.sleep(0.02 * (3 - device))  # later shards finish first
        with lock:
            seen[device] = sources.copy()
        return [(device, tuple(s)) for s in sources]

    monkeypatch.setattr(_shard, "_solve_on", fake_solve_on)
    src = np.arange(21, dtype=np.float64).reshape(7, 3)
    out = _shard.solve_sharded(object(), src, devices=[0, 1, 2])
    assert [s for _, s in out] == [tuple(s) for s in src]
    assert [d for d, _ in out] == [0, 0, 0, 1, 1, 2, 2]
    assert np.array_equal(np.concatenate([seen[d] for d in (0, 1, 2)]), src)
    # fewer sources than devices: one source per device, the rest idle
    out = _shard.solve_sharded(object(), src[:2], devices=[0, 1, 2])
    assert [d for d, _ in out] == [0, 1]

    def failing(device, *a):
        raise ValueError("source out of bound")

    with pytest.raises(ValueError, match="at most once"):
        _shard.solve_sharded(object(), src, devices=[0, 0])
    monkeypatch.setattr(_shard, "_solve_on", failing)
    with pytest.raises(ValueError, match="source out of bound"):
        _shard.solve_sharded(object(), src, devices=[0, 1])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _weights(nsrc, nrec, shape):
    """Seeded stand-in sensitivities: T[s, r] = sum(w[s, r] * velocity)."""
    return np.random.default_rng(1).uniform(0.1, 1.0, (nsrc, nrec) + shape)


def _fake_local_traveltimes(velocity, gridsize, sources, receivers, nsweep, memory_budget):
    """CPU stand-in for the device solve: differentiable in velocity, one row
    per source (its index in the full list is its first coordinate)."""
    shape = tuple(velocity.shape)
    w = torch.from_numpy(_weights(12, len(receivers), shape))
    rows = [w[int(s[0])] for s in sources]
    return torch.stack([(r * velocity).flatten(1).sum(1) for r in rows])


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    _shard._local_traveltimes = _fake_local_traveltimes
    shape = (3, 4, 5)
    v0 = torch.from_numpy(np.random.default_rng(0).uniform(1500, 2500, shape))
    src = np.column_stack([np.arange(7.0), np.zeros(7), np.zeros(7)])  # 7 sources
    rec = np.zeros((4, 3))
    v = v0.clone().requires_grad_(True)
    T, (lo, hi) = _shard.sharded_traveltimes(v, (1.0, 1.0, 1.0), src, rec, 2)
    loss = 0.5 * (T ** 2).sum()
    loss.backward()
    np.save(out + f".{rank}.npy", np.concatenate([[lo, hi], T.detach().numpy().ravel(),
                                                  v.grad.numpy().ravel()]))
    dist.destroy_process_group()


def test_two_ranks_split_sources_and_sum_the_gradient_in_rank_order(tmp_path):
    out = str(tmp_path / "rank")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    r0, r1 = np.load(out + ".0.npy"), np.load(out + ".1.npy")
    shape, nrec = (3, 4, 5), 4
    ncell = int(np.prod(shape))
    (lo0, hi0), (lo1, hi1) = r0[:2].astype(int), r1[:2].astype(int)
    assert (lo0, hi0, lo1, hi1) == (0, 4, 4, 7)
    n0, n1 = (hi0 - lo0) * nrec, (hi1 - lo1) * nrec
    T0, g0 = r0[2:2 + n0], r0[2 + n0:]
    T1, g1 = r1[2:2 + n1], r1[2 + n1:]
    # both ranks hold the same gradient bits: the sum of the two ranks'
    # gradients, rank 0's first
    assert np.array_equal(g0, g1) and len(g0) == ncell
    v0 = np.random.default_rng(0).uniform(1500, 2500, shape)
    w = _weights(12, nrec, shape)
    T = (w[:7] * v0).reshape(7, nrec, -1).sum(-1)
    assert np.allclose(np.concatenate([T0, T1]), T.ravel(), rtol=1e-14)
    local = [np.einsum("sr,srk->k", T[lo:hi], w[lo:hi].reshape(hi - lo, nrec, -1))
             for lo, hi in ((lo0, hi0), (lo1, hi1))]
    assert np.allclose(g0, local[0] + local[1], rtol=1e-12)
