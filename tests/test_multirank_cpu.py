"""The multi-GPU host path of bench.py on CPU ranks (gloo, world size 2).

Sources are independent solves, so N GPUs run N disjoint 256-source batches
with no collective on the data path (weak scaling); only the barrier and the
max-over-ranks timing touch the process group. Nothing here needs a GPU.
"""

import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    w, r = bench.dist_setup("gloo")
    assert (w, r) == (world, rank)
    src = torch.from_numpy(bench.rank_sources(rank))
    gathered = [torch.empty_like(src) for _ in range(world)]
    dist.all_gather(gathered, src)
    bench.barrier(world)
    t = bench.max_over_ranks(1.5 + rank, world)
    if rank == 0:
        np.save(out, np.stack([g.numpy() for g in gathered] + [np.full_like(src.numpy(), t)]))
    dist.destroy_process_group()


def test_two_ranks_shard_sources_and_take_the_max_time(tmp_path):
    out = str(tmp_path / "gathered.npy")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    a = np.load(out)
    s0, s1, t = a[0], a[1], a[2]
    # every rank solves its own 256 sources (weak scaling); rank 0's are the
    # single-GPU batch
    assert s0.shape == s1.shape == (256, 3)
    assert np.array_equal(s0, bench.surface_sources())
    assert not np.isin(s1.view("f8,f8,f8"), s0.view("f8,f8,f8")).any()
    ext = np.array(bench.SHAPE) * np.array(bench.D)
    assert np.all((s1 >= 0) & (s1 <= ext)) and np.all(s1[:, 0] == 0.0)
    assert np.all(t == 2.5)  # the max over ranks


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        steps, warmup = 1, 3

    assert bench.run_reference(Args) == 0
    assert capsys.readouterr().out == ""
