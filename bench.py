"""Benchmark of the 3D traveltime path on GB300: the batched many-source solve.

Workload (one step): a seeded layered float64 velocity model of 128 x 256 x 256
cells at 10 m (6 layers with uniform velocities in [1500, 4500] m/s, interfaces
perturbed by +-30 m of smoothed noise), 256 surface sources on a 16 x 16 grid
with seeded off-grid jitter, nsweep=2 with gradients, all solved by one
persistent kernel launch, then a-posteriori ray tracing from every source to
400 seeded surface receivers (102,400 rays).

Printed JSON line (rank 0):
  value     shots/s with the model, sources and receivers resident in HBM
  e2e       the same step through the drop-in Python API from host arrays
            (velocity upload, solve, rays and first-arrival picks copied back)
  plain     the same grid solved one source per launch (the "plain" solve)
  roofline  the sweep kernel's executed FP64 lane instructions per second
            against the FP64 pipe's peak measured in this run, with the
            reference's algorithmic operation count and the HBM rate beside it
  cpu_baseline  the reference's kernels on the host CPU (the oracle's C
            restatement, built for timing with the reference's numba
            floating-point licences, OpenMP over all host cores) on a bounded
            sample of the same workload

``--impl reference`` times that CPU implementation alone: numba is not
installed on these hosts, so the reference's kernels run as the oracle's C
restatement with all host threads (the reference's own pure-Python mode is
~1e4x slower still).
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "3D cell-updates/s & shots/s: batched vs plain GPU solve (FP64, rel err≤1e-12)"
SHAPE = (128, 256, 256)
D = (10.0, 10.0, 10.0)
NSRC = 256
NREC = 400
NSWEEP = 2
FLOP_PER_UPDATE = 160  # algorithmic FP64 operations of one 3D node update
BYTES_PER_UPDATE = 25  # slowness + tt read + tt write (8 B each) + 1 B branch record
# Per node update of the team sweep kernel on the layered benchmark model, from
# one ncu capture of that kernel on the 192-source 64x128x128 case: executed
# FP64 thread instructions (DADD + DMUL + DFMA, one per active lane) and DRAM
# bytes read + written. The bench scales both by the updates of the timed
# launch.
TEAM_FP64_LANE_OPS_PER_UPDATE = (31704945064 + 14876450935 + 12795162258) / 3221225472
TEAM_DRAM_BYTES_PER_UPDATE = (84846509568 + 8640589312) / 3221225472


def smooth2d(rng, shape, sigma):
    from scipy.ndimage import gaussian_filter

    p = gaussian_filter(rng.standard_normal(shape), sigma)
    p -= p.min()
    return 2.0 * p / p.max() - 1.0


def layered_model(shape=None, d=D, nlayers=6, seed=2024):
    """6 horizontal layers, seeded velocities in [1500, 4500] m/s, interfaces
    perturbed by +-30 m of smoothed noise."""
    shape = shape or SHAPE
    rng = np.random.default_rng(seed)
    nz, nx, ny = shape
    depth = nz * d[0]
    tops = np.sort(rng.uniform(0.1 * depth, 0.9 * depth, nlayers - 1))
    vels = rng.uniform(1500.0, 4500.0, nlayers)
    zc = (np.arange(nz) + 0.5) * d[0]
    layer = np.zeros(shape, dtype=np.int64)
    for t in tops:
        iface = t + 30.0 * smooth2d(rng, (nx, ny), 8.0)
        layer += zc[:, None, None] > iface[None, :, :]
    return vels[layer]


def surface_sources(shape=None, d=D, n_side=16, seed=7):
    shape = shape or SHAPE
    rng = np.random.default_rng(seed)
    ext = np.array(shape) * np.array(d)
    ix, iy = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="ij")
    x = (ix.ravel() + 0.5 + rng.uniform(-0.3, 0.3, n_side**2)) * ext[1] / n_side
    y = (iy.ravel() + 0.5 + rng.uniform(-0.3, 0.3, n_side**2)) * ext[2] / n_side
    return np.column_stack([np.zeros(n_side**2), x, y])


def surface_receivers(shape=None, d=D, n=NREC, seed=11):
    shape = shape or SHAPE
    rng = np.random.default_rng(seed)
    ext = (np.array(shape) - 0) * np.array(d)  # node extent = cells * spacing
    return np.column_stack(
        [np.zeros(n), rng.uniform(0.0, ext[1], n), rng.uniform(0.0, ext[2], n)]
    )


def updates_per_source(shape=None, nsweep=NSWEEP):
    shape = shape or SHAPE
    return 8 * nsweep * int(np.prod(shape))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = (
        "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[4:8]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": float(max(smax)) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def dist_setup(backend="nccl"):
    """One process per GPU (torchrun's RANK / LOCAL_RANK / WORLD_SIZE); gloo
    runs the same host logic on CPU ranks."""
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_sources(rank, shape=None):
    """The sources one rank solves: weak scaling gives every rank its own
    256-source batch, the jittered 16 x 16 surface grid seeded per rank (rank
    0 solves the single-GPU batch). Sources are independent solves
    (_fteik3d.py:508 prange), so no data moves between ranks."""
    return surface_sources(shape, seed=7 + 1000 * rank)


CPU_BUILD = ("the reference's kernels restated in C (numba is not installed on this host), "
             "built for timing with the reference's numba floating-point licences "
             "(gcc -O3, FMA contraction, reciprocal multiplication, no signed zeros), "
             "OpenMP over sources")


def cpu_sample(nthreads=None, nsrc=None, shape=None):
    """Time the CPU reference path (the oracle's timing build, all host cores,
    OpenMP over sources) on a bounded sample of the workload: as many sources
    as threads, solved with gradients, plus their rays. Returns (shots/s,
    threads, sample description)."""
    from oracle import oracle as O

    shape = shape or SHAPE
    nthreads = nthreads or os.cpu_count() or 1
    nsrc = nsrc or nthreads
    v = layered_model(shape)
    src = surface_sources(shape)[:nsrc]
    rec = surface_receivers(shape)
    O.lib(fast=True)
    t0 = time.perf_counter()
    tt, tg, vz = O.solve3d(1.0 / v, D, src, NSWEEP, True, nthreads=nthreads, fast=True)
    ax = O.axes(tt.shape[1:], D, np.zeros(3))
    max_dist = 2.0 * sum((n * h) ** 2 for n, h in zip(tt.shape[1:], D)) ** 0.5
    for s in range(nsrc):
        O.raytrace(ax, tg[s], rec, src[s], min(D), int(max_dist / min(D)), False, fast=True)
    dt = time.perf_counter() - t0
    desc = (f"{nsrc} of the {NSRC} sources on the {shape[0]}x{shape[1]}x{shape[2]} grid "
            f"(solve with gradients + {NREC} rays each), {nthreads} threads; {CPU_BUILD}")
    return nsrc / dt, nthreads, desc


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(nthreads)
    times = []
    for _ in range(args.steps):
        sps, _, desc = cpu_sample(nthreads)
        times.append(nthreads / sps)
    ms = 1e3 * float(np.mean(times))
    value = nthreads / (ms * 1e-3)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "shots/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded layered model, surface sources and receivers)",
        "config": workload_config(),
        "cell_updates_per_s": value * updates_per_source(),
        "cpu_baseline": {
            "value": value,
            "unit": "shots/s",
            "cores": nthreads,
            "kind": "port",
            "sample": desc,
        },
        "e2e": {"value": value, "unit": "shots/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def workload_config():
    return {
        "workload": f"batched 3D solve: {NSRC} surface sources on a "
                    f"{SHAPE[0]}x{SHAPE[1]}x{SHAPE[2]} layered model "
                    f"(dz=dx=dy=10 m), nsweep=2 with gradients, then {NSRC}x{NREC} rays",
        "grid": list(SHAPE),
        "sources": NSRC,
        "receivers_per_source": NREC,
        "nsweep": NSWEEP,
        "cell_updates_per_source": updates_per_source(),
        "l2": "inputs larger than L2 (%.1f GB of traveltimes per step)"
              % (NSRC * np.prod(np.array(SHAPE) + 1) * 8 / 1e9),
    }


def config1_models(shape=(200, 300), d=(10.0, 10.0), seed=1):
    """The plain 2D workload: v(z) = 1500 + 0.6 z (cell centres) times
    (1 + 0.1 p), p seeded N(0,1) noise Gaussian-smoothed with sigma = 8 cells
    and rescaled to [-1, 1]. Returns (v, v0 = the p = 0 model, source, d)."""
    from scipy.ndimage import gaussian_filter

    nz, nx = shape
    rng = np.random.default_rng(seed)
    p = gaussian_filter(rng.standard_normal((nz, nx)), 8.0)
    p = 2.0 * (p - p.min()) / (p.max() - p.min()) - 1.0
    zc = (np.arange(nz) + 0.5) * d[0]
    v0 = (1500.0 + 0.6 * zc)[:, None] * np.ones((nz, nx))
    return v0 * (1.0 + 0.1 * p), v0, np.array([5.3, 1234.7]), d


def linear_gradient_times(shape, d, src, v_top=1500.0, g=0.6, min_cells=5):
    """Analytic first-arrival times T = arccosh(1 + g^2 r^2 / (2 v_s v)) / g of
    the velocity v(z) = v_top + g z at the nodes of a grid (2D or 3D, z
    first), and the mask of nodes farther than ``min_cells`` cells from the
    source (the near-source nodes start from the solver's own analytic
    initialisation)."""
    axes = np.meshgrid(*[np.arange(n + 1) * h for n, h in zip(shape, d)], indexing="ij")
    r2 = sum((a - s) ** 2 for a, s in zip(axes, src))
    vs, vn = v_top + g * src[0], v_top + g * axes[0]
    t = np.arccosh(1.0 + g * g * r2 / (2.0 * vs * vn)) / g
    return t, r2 > (min_cells * min(d)) ** 2


def run_config1(args):
    """Plain 2D solve (the reference's CPU-runnable case): 200 x 300 cells at
    10 m, v(z) = 1500 + 0.6 z times (1 + 0.1 p), p seeded N(0,1) noise smoothed
    with sigma = 8 cells and rescaled to [-1, 1]; source (5.3, 1234.7), nsweep=2.
    Reports the GPU and CPU-oracle times, their parity, and the error of the
    p = 0 model against the analytic linear-gradient traveltime."""
    import torch

    import fteikpy_gb300 as fp
    from oracle import oracle as O

    import ctypes

    from fteikpy_gb300 import _device, _lib

    lib = _lib.load()
    v, v0, src, d = config1_models()
    eik = fp.Eikonal2D(v, d)

    def timed_solves():
        for _ in range(max(args.warmup, 1)):
            eik.solve(src, nsweep=2)
        torch.cuda.synchronize()
        ts = []
        for _ in range(max(args.steps, 1)):
            t0 = time.perf_counter()
            tt = eik.solve(src, nsweep=2)
            g = tt.grid
            ts.append(time.perf_counter() - t0)
        return ts, g

    lib.fteik_set_option(b"sweep2d_speculate", 0)
    times_nospec, g_nospec = timed_solves()
    lib.fteik_set_option(b"sweep2d_speculate", -1)
    lib.fteik_set_option(b"sweep2d_warp", 1)
    times_warp, g_warp = timed_solves()
    lib.fteik_set_option(b"sweep2d_warp", -1)
    times, g = timed_solves()
    nodes, hits = ctypes.c_ulonglong(), ctypes.c_ulonglong()
    _lib.check(lib.fteik2d_chain_stats(_device.ptr(_device.workspace("solve2d", 256)),
                                       ctypes.byref(nodes), ctypes.byref(hits),
                                       _device.stream()), "chain stats")
    tto, _, _ = O.solve2d(1.0 / v, d, [src], 2, False, nthreads=1)
    same = bool(np.array_equal(g, tto[0]))
    O.solve2d(1.0 / v, d, [src], 2, False, nthreads=1, fast=True)
    t0 = time.perf_counter()
    O.solve2d(1.0 / v, d, [src], 2, False, nthreads=1, fast=True)
    cpu = time.perf_counter() - t0
    # analytic linear-gradient traveltime for p = 0 (velocity at cell centres)
    t_lin = fp.Eikonal2D(v0, d).solve(src, nsweep=2).grid
    t_ana, far = linear_gradient_times(v.shape, d, src)
    rel = np.abs(t_lin - t_ana)[far] / t_ana[far]
    print(json.dumps({
        "config": 1,
        "metric": "2D plain solve time (200x300, nsweep=2, one off-grid source)",
        "value": 1e3 * float(np.median(times)), "unit": "ms", "higher_is_better": False,
        "cpu_baseline": {"value": 1e3 * cpu, "unit": "ms", "cores": 1, "kind": "port",
                         "sample": "the same solve, 1 thread; " + CPU_BUILD},
        "parity_bitwise_vs_oracle": same and bool(np.array_equal(g_nospec, g))
                                    and bool(np.array_equal(g_warp, g)),
        "speculation": {"node_updates": nodes.value, "hits": hits.value,
                        "hit_fraction": hits.value / max(nodes.value, 1),
                        "ms_without": 1e3 * float(np.median(times_nospec))},
        "ms_one_warp": 1e3 * float(np.median(times_warp)),
        "analytic_linear_gradient_rel_err": {"max": float(rel.max()), "median": float(np.median(rel)),
                                             "excluding": "nodes within 5 cells of the source"},
        "note": "the reference's 2D sweep is one serial dependence chain; a single 2D source "
                "runs on a block of 4 warps: three warps precompute each pass's terms that "
                "do not depend on the previous node, and each row's whole update with the "
                "previous node's value from before the pass, ahead of one lane that runs the "
                "chain, taking the precomputed update where the actual value has the same "
                "bits (ms_one_warp: one warp doing both in turn)",
    }))
    return 0


def run_config2(args):
    """Plain 3D solve: one seeded off-grid surface source on the 150 x 200 x 200
    layered model at 10 m, nsweep=2 with gradients, then traveltimes at 10,000
    seeded points and 400 rays to seeded surface receivers, through the drop-in
    API (results copied to the host)."""
    import torch

    import fteikpy_gb300 as fp
    from oracle import oracle as O

    shape = (150, 200, 200)
    v = layered_model(shape)
    rng = np.random.default_rng(2)
    ext = np.array(shape) * np.array(D)
    src = np.array([0.0, rng.uniform(0.2, 0.8) * ext[1], rng.uniform(0.2, 0.8) * ext[2]])
    pts = rng.uniform([0.0, 0.0, 0.0], ext, (10000, 3))
    rec = np.column_stack([np.zeros(NREC), rng.uniform(0, ext[1], NREC), rng.uniform(0, ext[2], NREC)])
    eik = fp.Eikonal3D(v, D)

    def step():
        tt = eik.solve(src, nsweep=NSWEEP, return_gradient=True)
        a = tt(pts)
        rays = tt.raytrace(rec)
        return tt, a, rays

    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize()
    times = []
    for _ in range(max(args.steps, 1)):
        t0 = time.perf_counter()
        tt, a, rays = step()
        times.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    tto, tgo, vzo = O.solve3d(1.0 / v, D, [src], NSWEEP, True)
    ax = O.axes(tto.shape[1:], D, np.zeros(3))
    ao = O.vinterp(ax, tto[0], pts, src, vzo[0])
    max_dist = 2.0 * sum((n * h) ** 2 for n, h in zip(tto.shape[1:], D)) ** 0.5
    rays_o = O.raytrace(ax, tgo[0], rec, src, min(D), int(max_dist / min(D)), False)
    cpu = time.perf_counter() - t0
    same = bool(np.array_equal(tt.grid, tto[0]) and np.array_equal(a, ao)
                and all(np.array_equal(x, y) for x, y in zip(rays, rays_o)))
    print(json.dumps({
        "config": 2,
        "metric": "plain 3D solve + 10,000 traveltime queries + 400 rays (150x200x200, nsweep=2)",
        "value": 1e3 * float(np.median(times)), "unit": "ms", "higher_is_better": False,
        "cell_updates_per_s": updates_per_source(shape) / float(np.median(times)),
        "cpu_baseline": {"value": 1e3 * cpu, "unit": "ms", "cores": os.cpu_count(), "kind": "port",
                         "sample": "the same step with the C oracle (the solve is one source: 1 thread)"},
        "parity_bitwise_vs_oracle": same,
    }))
    return 0


def uneven_models(nmodel=64, seed=44, sizes=(32, 160)):
    """Config-4 batch: per model, cell counts drawn uniformly from [32, 160]
    per axis (``sizes``), one grid spacing drawn from [5, 20] m, velocity
    1500..2500 m/s at the top plus a 0.3..1.0 1/s gradient, times (1 + 0.1 p)
    with p seeded normal noise Gaussian-smoothed (sigma 3 cells) and rescaled
    to [-1, 1], and 1..16 seeded off-grid sources anywhere in the model."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nmodel):
        shape = tuple(int(x) for x in rng.integers(sizes[0], sizes[1] + 1, 3))
        d = (float(rng.uniform(5.0, 20.0)),) * 3
        z = (np.arange(shape[0]) + 0.5) * d[0]
        v = (rng.uniform(1500.0, 2500.0) + rng.uniform(0.3, 1.0) * z)[:, None, None]
        p = gaussian_filter(rng.standard_normal(shape), 3.0)
        p -= p.min()
        p = 2.0 * p / p.max() - 1.0
        v = v * (1.0 + 0.1 * p)
        ext = np.array(shape) * np.array(d)
        src = rng.uniform(0.02, 0.98, (int(rng.integers(1, 17)), 3)) * ext
        out.append((v, d, src))
    return out


def run_config4(args):
    """Batched uneven models: 64 models of seeded sizes and spacings with 1-16
    sources each, all solved (nsweep=2) by one persistent sweep launch with
    the launch shape picked by the autotuner; beside it the same work as one
    Eikonal3D.solve per model (64 launches) and the C oracle on a sample."""
    import torch

    import fteikpy_gb300 as fp
    from fteikpy_gb300 import _lib
    from oracle import oracle as O

    cases = uneven_models()
    solvers = [fp.Eikonal3D(v, d) for v, d, _ in cases]
    sources = [s for _, _, s in cases]
    nsrc = sum(len(s) for s in sources)
    updates = sum(8 * NSWEEP * int(np.prod(v.shape)) * len(s) for v, _, s in cases)
    lib = _lib.load()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, steps):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    batch = lambda: fp.solve_batch(solvers, sources, nsweep=NSWEEP)  # noqa: E731
    lib.fteik_clear_tuning()
    default_ms = timed(batch, max(args.steps, 1))
    q0 = time.perf_counter()
    shape = fp.autotune(solvers, sources)
    tune_s = time.perf_counter() - q0
    for _ in range(max(args.warmup - 1, 0)):
        batch()
    tuned_ms = timed(batch, max(args.steps, 1))

    def plain():
        return [eik.solve(src, nsweep=NSWEEP) for eik, src in zip(solvers, sources)]

    plain_ms = timed(plain, max(args.steps, 1))
    out = batch()
    ref = plain()
    same_as_plain = all(
        all(np.array_equal(a.grid, b.grid) for a, b in zip(x, y)) for x, y in zip(out, ref)
    )
    # the C oracle on a sample of models (all host threads, parallel over sources)
    sample = list(range(0, len(cases), 16))
    q0 = time.perf_counter()
    oracle_tt = [O.solve3d(1.0 / cases[m][0], cases[m][1], cases[m][2], NSWEEP, False)[0]
                 for m in sample]
    cpu_s = time.perf_counter() - q0
    sample_updates = sum(8 * NSWEEP * int(np.prod(cases[m][0].shape)) * len(cases[m][2])
                         for m in sample)
    same_as_oracle = all(
        np.array_equal(np.stack([t.grid for t in out[m]]), tt) for m, tt in zip(sample, oracle_tt)
    )
    print(json.dumps({
        "config": 4,
        "metric": "uneven 3D batch: 64 models (32-160 cells/axis, 5-20 m spacing), 1-16 sources each, nsweep=2",
        "value": 1e3 * nsrc / tuned_ms, "unit": "shots/s", "higher_is_better": True,
        "cell_updates_per_s": updates / (tuned_ms * 1e-3),
        "ms_per_batch": tuned_ms, "ms_per_batch_default_shape": default_ms,
        "autotune": dict(shape, seconds=tune_s),
        "plain_one_solve_per_model": {"ms": plain_ms, "shots_per_s": 1e3 * nsrc / plain_ms,
                                      "launches": len(cases)},
        "batch_over_plain": plain_ms / tuned_ms,
        "models": len(cases), "sources": nsrc, "cell_updates": updates,
        "bitwise_vs_per_model_solves": bool(same_as_plain),
        "bitwise_vs_oracle_sample": bool(same_as_oracle),
        "cpu_baseline": {"value": sample_updates / cpu_s, "unit": "cell-updates/s",
                         "cores": os.cpu_count(), "kind": "port",
                         "sample": f"models {sample} with the C oracle"},
    }))
    return 0


def tomography_models(shape=(96, 128, 128), d=D, seed=5):
    """Linear-gradient starting model v(z) = 1500 + 0.6 z and the true model:
    the same times (1 + 0.08 exp(-r^2 / (2 * 150 m^2))), a Gaussian anomaly of
    radius 150 m centred at a seeded point in the middle of the grid."""
    rng = np.random.default_rng(seed)
    ext = np.array(shape) * np.array(d)
    zc, xc, yc = [(np.arange(n) + 0.5) * h for n, h in zip(shape, d)]
    v0 = (1500.0 + 0.6 * zc)[:, None, None] * np.ones(shape)
    c = ext * rng.uniform([0.4, 0.35, 0.35], [0.6, 0.65, 0.65])
    r2 = ((zc - c[0])[:, None, None] ** 2 + (xc - c[1])[None, :, None] ** 2
          + (yc - c[2])[None, None, :] ** 2)
    return v0, v0 * (1.0 + 0.08 * np.exp(-r2 / (2.0 * 150.0**2)))


def tie_broken(v, rel=1e-3, seed=17):
    """``v`` with every cell's velocity times (1 + rel u), u seeded uniform in
    [-1, 1]: on a linear-gradient model this breaks the exact ties between
    laterally neighbouring cells that the solver's slowness minima take."""
    return v * (1.0 + rel * np.random.default_rng(seed).uniform(-1.0, 1.0, v.shape))


def oracle_receiver_times(O, v, src, rec, nsweep=NSWEEP, probe=False, margin=0.0):
    """[nsrc, nrec] apparent-velocity traveltimes through the oracle; with
    ``probe`` also the per-source decision digests and the near-tied cells."""
    if probe:
        tt, vz, dig, tied = O.solve3d_probe(1.0 / v, D, src, nsweep, margin=margin)
    else:
        tt, _, vz = O.solve3d(1.0 / v, D, src, nsweep, False)
        dig = tied = None
    ax = O.axes(tt.shape[1:], D, np.zeros(3))
    T = np.stack([O.vinterp(ax, tt[s], rec, src[s], vz[s]) for s in range(len(src))])
    return T, dig, tied


FD_STEP = 1e-6    # relative step of the central differences
TIE_MARGIN = 4e-6  # relative margin a slowness minimum needs to count as untied


def fd_check(O, v, src, rec, t_obs, g, ncells, tie_free, min_frac, seed=3):
    """Central differences (relative step 1e-6) of 0.5 sum (T - t_obs)^2 through
    the oracle's solve, against the gradient ``g``, on seeded cells whose
    |g| is at least ``min_frac`` of the largest.

    With ``tie_free`` a cell qualifies only away from the solver's branch
    ties: no slowness minimum taken by a kept operator may have another cell
    within TIE_MARGIN of it (oracle probe at ``v``), and every decision of
    the sweeps (candidate kept, cells attaining each minimum) must be the same
    at v + h and v - h as at v (oracle decision digests); candidates that
    fail are skipped and counted. Returns a dict of the statistics."""
    shape = v.shape
    gmax = float(np.abs(g).max())
    _, dig0, tied = oracle_receiver_times(O, v, src, rec, probe=True, margin=TIE_MARGIN)
    pool = np.flatnonzero(np.abs(g.ravel()) >= min_frac * gmax)
    significant = len(pool)
    if tie_free:
        pool = pool[~tied.ravel()[pool]]
    order = np.random.default_rng(seed).permutation(pool)
    errs, rejected = [], 0
    for c in order:
        if len(errs) >= ncells:
            break
        idx = np.unravel_index(c, shape)
        h = FD_STEP * v[idx]
        vp = v.copy()
        vp[idx] += h
        vm = v.copy()
        vm[idx] -= h
        tp, dp, _ = oracle_receiver_times(O, vp, src, rec, probe=tie_free, margin=TIE_MARGIN)
        tm, dm, _ = oracle_receiver_times(O, vm, src, rec, probe=tie_free, margin=TIE_MARGIN)
        if tie_free and not (np.array_equal(dp, dig0) and np.array_equal(dm, dig0)):
            rejected += 1
            continue
        # L(v+h) - L(v-h) summed term by term as 0.5 (tp - tm)(tp + tm - 2 t_obs):
        # the same difference without cancelling two losses ~1e8 times larger
        fd = float(np.sum(0.5 * (tp - tm) * (tp + tm - 2.0 * t_obs))) / (2.0 * h)
        errs.append(abs(fd - g[idx]) / abs(fd))
    errs = np.array(errs)
    return {
        "cells": int(len(errs)),
        "significant_cells": int(significant),
        "eligible_cells": int(len(pool)),
        "rejected_decision_change": int(rejected) if tie_free else None,
        "min_abs_grad_over_max": min_frac,
        "rel_err_median": float(np.median(errs)) if len(errs) else None,
        "rel_err_p90": float(np.quantile(errs, 0.9)) if len(errs) else None,
        "rel_err_max": float(errs.max()) if len(errs) else None,
        "cells_within_1e-6": int((errs <= 1e-6).sum()),
        "cells_within_1e-4": int((errs <= 1e-4).sum()),
    }


def run_fd_cpu(args):
    """The finite-difference checks of --config 5 on the host alone: the
    gradient is the oracle's sequential reverse-mode adjoint, which the GPU
    gradient equals to about 2e-15 of its largest entry on this problem (the
    GPU run of --config 5 and tests/test_gpu_configs.py check that on every
    cell), and the central differences go through the oracle's solve as in
    --config 5. The GPU's time is not spent on the host's finite differences."""
    from oracle import oracle as O

    shape = (48, 64, 64) if args.small else (96, 128, 128)
    v0, vt = tomography_models(shape)
    src = surface_sources(shape, n_side=4 if args.small else 8, seed=7)
    rec = surface_receivers(shape, n=NREC, seed=11)
    t_obs = oracle_receiver_times(O, vt, src, rec)[0]

    def gradient(v):
        T = oracle_receiver_times(O, v, src, rec)[0]
        s = 1.0 / v
        return -O.adjoint3d(s, D, src, NSWEEP, rec, T - t_obs) * s * s

    q0 = time.perf_counter()
    vb = tie_broken(v0)
    tie_free = fd_check(O, vb, src, rec, t_obs, gradient(vb), args.fd_cells, True, 1e-2)
    tie_free["model"] = ("the start model with every cell's velocity times (1 + 1e-3 u), u "
                         "seeded uniform in [-1, 1]")
    tie_free["selection"] = ("seeded; |grad| >= 1e-2 max|grad|; no kept operator's slowness "
                             "minimum has a second cell within 4e-6 of it; the sweeps' "
                             "decisions (oracle digests) identical at v - h, v, v + h")
    g0 = gradient(v0)
    start = fd_check(O, v0, src, rec, t_obs, g0, args.fd_cells, False, 1e-4)
    _, _, tied0 = oracle_receiver_times(O, v0, src, rec, probe=True, margin=TIE_MARGIN)
    pool0 = np.flatnonzero(np.abs(g0.ravel()) >= 1e-4 * np.abs(g0).max())
    start["tie_free_significant_cells"] = int((~tied0.ravel()[pool0]).sum())
    start["selection"] = "seeded, |grad| >= 1e-4 max|grad| (ties included)"
    print(json.dumps({
        "config": 5,
        "metric": "finite-difference check of d(loss)/d(velocity), %dx%dx%d, %d sources x 400 "
                  "receivers, nsweep=2" % (shape + (len(src),)),
        "gradient": "the oracle's reverse-mode adjoint (equal to the GPU gradient to ~2e-15 "
                    "of its largest entry)",
        "fd": {"rel_step": FD_STEP, "cells_within_1e-6": tie_free["cells_within_1e-6"],
               "tie_free": tie_free, "start_model": start},
        "host_seconds": time.perf_counter() - q0, "threads": os.cpu_count(),
    }))
    return 0


def run_config5(args):
    """Adjoint gradient for tomography: 96 x 128 x 128 at 10 m, 64 surface
    sources x 400 surface receivers, loss = 0.5 sum((T_pred - T_obs)^2) with
    T_obs from the true model; forward and adjoint through the autograd
    function, the gradient checked by central differences (relative step 1e-6)
    on 50 seeded cells through the C oracle: on cells away from the solver's
    branch ties of the start model with its lateral ties broken, and on
    |grad|-selected cells of the exact start model."""
    import torch

    import fteikpy_gb300 as fp
    from fteikpy_gb300 import _adjoint, _lib
    from fteikpy_gb300._solver import solve3d_device
    from oracle import oracle as O

    if args.adj_shape:
        shape = tuple(int(x) for x in args.adj_shape.split(","))
    else:
        shape = (48, 64, 64) if args.small else (96, 128, 128)
    n_side = int(round(np.sqrt(args.adj_sources))) if args.adj_sources else (4 if args.small else 8)
    v0, vt = tomography_models(shape)
    src = surface_sources(shape, n_side=n_side, seed=7)
    rec = surface_receivers(shape, n=NREC, seed=11)
    dev = torch.device("cuda", 0)
    budget = int(args.memory_budget * 1e9) if args.memory_budget else None
    t_obs = fp.traveltimes(torch.tensor(vt, device=dev), D, src, rec, NSWEEP, budget).detach()
    vel = torch.tensor(v0, device=dev)

    def fwd_plain():
        slow = 1.0 / vel
        return solve3d_device(slow, D, src, NSWEEP, False)[0]

    def step(v=vel):
        x = v.clone().requires_grad_(True)
        T = fp.traveltimes(x, D, src, rec, NSWEEP, budget)
        loss = 0.5 * ((T - t_obs) ** 2).sum()
        e_mid.record()
        loss.backward()
        return x.grad, loss, T

    e0, e_mid, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    for _ in range(max(args.warmup, 1)):
        fwd_plain()
        step()
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats(dev)
    base_mem = torch.cuda.memory_allocated(dev)
    plain_ms, fwd_ms, bwd_ms = [], [], []
    for _ in range(max(args.steps, 1)):
        e0.record()
        fwd_plain()
        e1.record()
        torch.cuda.synchronize()
        plain_ms.append(e0.elapsed_time(e1))
        e0.record()
        g, loss, T = step()
        e1.record()
        torch.cuda.synchronize()
        fwd_ms.append(e0.elapsed_time(e_mid))
        bwd_ms.append(e_mid.elapsed_time(e1))
    peak_mem = torch.cuda.max_memory_allocated(dev) - base_mem
    lib = _lib.load()
    used_budget = budget if budget is not None else int(
        _adjoint.BUDGET_SHARE * torch.cuda.mem_get_info(dev)[0])
    chunk, group, _ = _adjoint._chunk_plan(lib, shape, len(src), NSWEEP, used_budget)
    g = g.cpu().numpy()
    T = T.detach().cpu().numpy()
    t_obs_h = t_obs.cpu().numpy()
    plain, fwd, bwd = (float(np.median(x)) for x in (plain_ms, fwd_ms, bwd_ms))
    line = {
        "config": 5,
        "metric": "adjoint d(loss)/d(velocity), %dx%dx%d, %d sources x 400 receivers, nsweep=2"
                  % (shape + (len(src),)),
        "value": fwd + bwd, "unit": "ms", "higher_is_better": False,
        "forward_plain_ms": plain, "forward_with_tape_ms": fwd, "adjoint_ms": bwd,
        "adjoint_over_forward": bwd / plain, "forward_plus_adjoint_over_forward": (fwd + bwd) / plain,
        "memory": {"peak_bytes_above_inputs": int(peak_mem), "budget_bytes": used_budget,
                   "sources_per_chunk": chunk, "sources_per_reverse_group": group,
                   "tape_bytes_per_node_source": lib.fteik3d_tape_bytes(*shape, 1, NSWEEP, 2)
                   / float(np.prod(np.array(shape) + 1))},
    }
    if not args.no_cpu:
        # CPU: the oracle's forward and its sequential reverse-mode adjoint,
        # which the GPU gradient must equal on every cell
        q0 = time.perf_counter()
        t_oracle = oracle_receiver_times(O, v0, src, rec)[0]
        cpu_fwd = time.perf_counter() - q0
        q0 = time.perf_counter()
        s0 = 1.0 / v0
        g_oracle = -O.adjoint3d(s0, D, src, NSWEEP, rec, t_oracle - t_obs_h) * s0 * s0
        cpu_adj = time.perf_counter() - q0
        gmax = float(np.abs(g).max())
        line["forward_bitwise_vs_oracle"] = bool(np.array_equal(T, t_oracle))
        line["adjoint_vs_oracle_adjoint_max_abs_over_gmax"] = float(np.abs(g - g_oracle).max() / gmax)
        line["cpu_baseline"] = {"value": 1e3 * (cpu_fwd + cpu_adj), "unit": "ms",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "one forward + adjoint with the C oracle "
                                          "(OpenMP over sources)",
                                "forward_ms": 1e3 * cpu_fwd, "adjoint_ms": 1e3 * cpu_adj}
    if args.fd_cells > 0:
        # 1. away from branch ties: the start model with its lateral ties
        #    broken (each cell within 0.1%), cells whose slowness minima are
        #    untied and whose sweeps decide alike at v +- h; derivatives of at
        #    least 1% of the largest (below that the rounding of the
        #    traveltimes, about 4e-10 of the largest derivative in the
        #    central difference, passes 1e-6 of the cell's own)
        vb = tie_broken(v0)
        gb = step(torch.tensor(vb, device=dev))[0].cpu().numpy()
        tie_free = fd_check(O, vb, src, rec, t_obs_h, gb, args.fd_cells, True, 1e-2)
        tie_free["model"] = ("the start model with every cell's velocity times (1 + 1e-3 u), u "
                             "seeded uniform in [-1, 1]")
        tie_free["selection"] = ("seeded; |grad| >= 1e-2 max|grad|; no kept operator's slowness "
                                 "minimum has a second cell within 4e-6 of it; the sweeps' "
                                 "decisions (oracle digests) identical at v - h, v, v + h")
        # 2. the exact start model: how many significant cells are tie-free,
        #    and the |grad|-selected cells, ties included
        start = fd_check(O, v0, src, rec, t_obs_h, g, args.fd_cells, False, 1e-4)
        _, _, tied0 = oracle_receiver_times(O, v0, src, rec, probe=True, margin=TIE_MARGIN)
        pool0 = np.flatnonzero(np.abs(g.ravel()) >= 1e-4 * np.abs(g).max())
        start["tie_free_significant_cells"] = int((~tied0.ravel()[pool0]).sum())
        start["selection"] = "seeded, |grad| >= 1e-4 max|grad| (ties included)"
        line["fd"] = {"rel_step": FD_STEP, "cells_within_1e-6": tie_free["cells_within_1e-6"],
                      "tie_free": tie_free, "start_model": start}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--plain-sources", type=int, default=8,
                    help="sources solved one per launch for the plain leg")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end API timing")
    ap.add_argument("--no-plain", action="store_true", help="skip the one-source-per-launch timing")
    ap.add_argument("--config", type=int, default=3, choices=[1, 2, 3, 4, 5],
                    help="1: plain 2D solve, 2: plain 3D solve + queries + rays, 3: batched "
                         "(default), 4: uneven multi-model batch, 5: adjoint gradient")
    ap.add_argument("--fd-cells", type=int, default=50,
                    help="cells of the finite-difference check of --config 5")
    ap.add_argument("--fd-cpu", action="store_true",
                    help="--config 5: only the finite-difference checks, on the host, with the "
                         "oracle's adjoint as the gradient")
    ap.add_argument("--adj-shape", default=None,
                    help="--config 5: grid cells nz,nx,ny (default 96,128,128)")
    ap.add_argument("--adj-sources", type=int, default=0,
                    help="--config 5: sources on a square surface grid (default 64)")
    ap.add_argument("--memory-budget", type=float, default=0.0,
                    help="--config 5: device GB the tapes and workspaces may take "
                         "(default: 80%% of the free memory)")
    ap.add_argument("--small", action="store_true",
                    help="profiling case: 192 sources on a 64x128x128 grid (1.7 GB of traveltimes, "
                         "> L2; 108K items per sweep, so the same team kernel as the full step); "
                         "with --config 5: 16 sources on 48x64x64")
    ap.add_argument("--option", action="append", default=[], metavar="NAME=VALUE",
                    help="library tuning knob (fteik_set_option), e.g. adjoint_chunk=4; "
                         "results are identical for every setting")
    args = ap.parse_args()
    if args.option and args.impl != "reference":
        from fteikpy_gb300 import _lib

        for item in args.option:
            name, value = item.split("=", 1)
            _lib.check(_lib.load().fteik_set_option(name.encode(), int(value)), "option " + name)
    if args.small:
        global SHAPE, NSRC
        SHAPE, NSRC = (64, 128, 128), 192
    if args.impl == "reference":
        return run_reference(args)
    if args.config == 5 and args.fd_cpu:
        return run_fd_cpu(args)
    if args.config in (1, 2, 4, 5):
        import torch

        if torch.cuda.is_available():
            torch.cuda.set_device(0)
        return {1: run_config1, 2: run_config2, 4: run_config4, 5: run_config5}[args.config](args)

    import torch

    import fteikpy_gb300 as fp
    from fteikpy_gb300 import _device, _lib, _solver
    from fteikpy_gb300._grid import trace_rays_device

    world, rank = dist_setup()
    lib = _lib.load()
    dev = _device.device()

    v = layered_model()
    src = rank_sources(rank)[:NSRC]
    rec = surface_receivers()
    nz, nx, ny = SHAPE
    node_shape = (nz + 1, nx + 1, ny + 1)
    axes = [_device.to_device(a) for a in
            [np.arange(n) * h for n, h in zip(node_shape, D)]]
    max_dist = 2.0 * sum((n * h) ** 2 for n, h in zip(node_shape, D)) ** 0.5
    max_step = int(max_dist / min(D))

    # resident inputs
    slow = _device.slowness(_device.to_device(v))
    ends = _device.to_device(np.tile(rec, (NSRC, 1)))
    gidx = torch.arange(NSRC, dtype=torch.int32, device=dev).repeat_interleave(NREC)
    src_dev = _device.to_device(src)
    grad_stride = int(np.prod(node_shape)) * 3

    lib.fteik_kernel_timing(1)
    sweep_ms = []

    def step():
        tt, tg, vz = _solver.solve3d_device(slow, D, src, NSWEEP, True)
        ms = __import__("ctypes").c_float()
        lib.fteik_last_sweep_ms(ms)
        sweep_ms.append(ms.value)
        packed, lengths = trace_rays_device(3, axes, tg, gidx, ends, src_dev, min(D), max_step,
                                            False, grad_stride)
        return tt, tg, packed

    for _ in range(args.warmup):
        out = step()
        del out
    torch.cuda.synchronize()
    sweep_ms.clear()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        out = step()
        del out
    e1.record()
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms_step = max_over_ranks(e0.elapsed_time(e1) / args.steps, world)
    shots = NSRC * world / (ms_step * 1e-3)
    sweep = float(np.mean(sweep_ms))

    # roofline of the sweep kernel (one launch = all sweeps of all sources).
    # The FP64 pipe's peak is measured in this run by a DFMA loop
    # (fteik_fp64_peak, 2 flops per DFMA lane); in FP64 lane instructions per
    # second it is half that. The kernel's executed lane instructions per
    # update come from an ncu capture of the same kernel (see the constant).
    kernel_name = lib.fteik_last_sweep_kernel().decode()
    updates = updates_per_source() * NSRC
    scratch = torch.empty(152 * 8 * 256, dtype=torch.float64, device=dev)
    peak = __import__("ctypes").c_double()
    lib.fteik_fp64_peak(_device.ptr(scratch), 152 * 8, 20000, peak, _device.stream())
    peak_lane_ops = peak.value / 2.0
    executed_lane_ops = updates * TEAM_FP64_LANE_OPS_PER_UPDATE / (sweep * 1e-3)
    algorithmic_ops = updates * FLOP_PER_UPDATE / (sweep * 1e-3)
    hbm_gbs = updates * BYTES_PER_UPDATE / (sweep * 1e-3) / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm_peak = json.load(open(peaks_path))["hbm_gbs"] if os.path.exists(peaks_path) else 6800.0
    traffic = TEAM_DRAM_BYTES_PER_UPDATE * updates

    # plain: one source per launch on the same grid, each with its 400 rays,
    # timed with CUDA events on the launching stream
    plain_n = 0 if args.no_plain else args.plain_sources
    plain_ms = None
    if plain_n:
        rec_dev = _device.to_device(rec)
        tt1, tg1, _ = _solver.solve3d_device(slow, D, src[:1], NSWEEP, True)  # warm
        del tt1, tg1
        torch.cuda.synchronize()
        pe0 = torch.cuda.Event(enable_timing=True)
        pe1 = torch.cuda.Event(enable_timing=True)
        pe0.record()
        for s in range(plain_n):
            tt1, tg1, _ = _solver.solve3d_device(slow, D, src[s:s + 1], NSWEEP, True)
            trace_rays_device(3, axes, tg1, None, rec_dev, src_dev[s:s + 1], min(D), max_step,
                              False)
            del tt1, tg1
        pe1.record()
        torch.cuda.synchronize()
        plain_ms = pe0.elapsed_time(pe1) / plain_n
    plain_shots = 1e3 / plain_ms if plain_n else None

    # e2e through the drop-in API from host arrays
    h2d = v.nbytes + src.nbytes + rec.nbytes * NSRC
    d2h = [0]

    def e2e_step():
        eik = fp.Eikonal3D(v, D)
        tts = eik.solve(src, nsweep=NSWEEP, return_gradient=True)
        nb = 0
        for t in tts:
            rays = t.raytrace(rec)
            picks = t(rec)
            nb += sum(r.nbytes for r in rays) + picks.nbytes
        d2h[0] = nb
        return tts

    e2e_shots = None
    if not args.no_e2e and args.e2e_steps > 0:
        e2e_step()
        torch.cuda.synchronize()
        barrier(world)
        q0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        torch.cuda.synchronize()
        barrier(world)
        e2e_ms = max_over_ranks(1e3 * (time.perf_counter() - q0) / args.e2e_steps, world)
        e2e_shots = NSRC * world / (e2e_ms * 1e-3)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sps, cores, desc = cpu_sample()
        cpu = {"value": sps, "unit": "shots/s", "cores": cores, "kind": "port", "sample": desc}

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": shots,
            "unit": "shots/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic (seeded layered model, surface sources and receivers)",
            "config": workload_config(),
            "cell_updates_per_s": shots * updates_per_source(),
            "plain": {
                "value": plain_shots,
                "unit": "shots/s",
                "ms_per_shot": plain_ms,
                "sources": plain_n,
                "what": "same grid, one source per solve launch (+ its 400 rays), CUDA events",
                "batched_over_plain": (shots / world / plain_shots) if plain_shots else None,
            },
            "roofline": {
                "bound": "fp64",
                "kernel": kernel_name,
                "unit": "T FP64 lane-instructions/s",
                "achieved": executed_lane_ops / 1e12,
                "peak": peak_lane_ops / 1e12,
                "frac": executed_lane_ops / peak_lane_ops,
                "executed_lane_ops_per_update": TEAM_FP64_LANE_OPS_PER_UPDATE,
                "executed_source": "ncu sm__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on "
                                   "of this kernel on the 192-source 64x128x128 layered case, "
                                   "per node update, times the updates of this launch",
                "peak_source": "DFMA loop measured in this run (fteik_fp64_peak): "
                               "%.4f TFLOP/s counting 2 flops per DFMA lane, i.e. %.4f T "
                               "lane-instructions/s" % (peak.value / 1e12, peak_lane_ops / 1e12),
                "algorithmic": {
                    "ops_per_update": FLOP_PER_UPDATE,
                    "achieved": algorithmic_ops / 1e12,
                    "unit": "T ops/s (each IEEE add, mul, compare, sqrt, div of the "
                            "reference's update counted once)",
                    "over_lane_instruction_peak": algorithmic_ops / peak_lane_ops,
                    "note": "above 1 because the kernel runs fewer FP64 instructions than "
                            "the reference's operation count: comparisons run on the integer "
                            "pipe and operators of nodes that provably keep their value are "
                            "skipped (exact, bitwise-tested)",
                },
                "kernel_ms": sweep,
                "hbm": {"achieved": hbm_gbs, "peak": hbm_peak, "unit": "GB/s",
                        "frac": hbm_gbs / hbm_peak, "bytes_per_update": BYTES_PER_UPDATE},
                "traffic": traffic,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of this "
                                  "kernel on the 192-source 64x128x128 case, per node update, "
                                  "times the updates of this launch",
            },
            "e2e": {
                "value": e2e_shots,
                "unit": "shots/s",
                "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h[0]),
                "what": "Eikonal3D(host velocity).solve(256 sources, gradients) + "
                        "raytrace and picks per source through the drop-in API",
            },
            # per step: pencil order, coefficients, fill, init, sweep and gradient
            # kernels of the solve, then the ray and ray-pack kernels
            "gpu_launches": 8 * args.steps,
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
