"""The CUDA adjoint of the 3D solve (``fteik3d_solve_tape`` +
``fteik3d_adjoint`` behind ``fteikpy_gb300.traveltimes``) against the oracle.

Two references: the oracle's sequential reverse-mode adjoint (its own test
file pins it to finite differences), compared on every cell; and central
finite differences taken through the oracle's solve directly. The loss is
0.5 * sum((T - T_obs)^2) over all source-receiver pairs, T the
apparent-velocity interpolated traveltime at the receivers.
"""

import numpy as np
import pytest
import torch

import fteikpy_gb300 as fp
from oracle import oracle as O
from adjoint_cases import (
    D,
    central_difference,
    check_cells,
    geometry,
    oracle_times,
    oracle_velocity_gradient,
    velocity,
)

pytestmark = pytest.mark.gpu


def gpu_gradient(v0, src, rec, nsweep, t_obs, memory_budget=None):
    vt = torch.tensor(v0, device="cuda", requires_grad=True)
    T = fp.traveltimes(vt, D, src, rec, nsweep, memory_budget)
    loss = 0.5 * ((T - torch.as_tensor(t_obs, device="cuda")) ** 2).sum()
    loss.backward()
    return T.detach().cpu().numpy(), vt.grad.cpu().numpy()


@pytest.mark.parametrize(
    "shape,nsweep,perturb",
    [((12, 14, 16), 1, True), ((12, 14, 16), 2, True), ((12, 14, 16), 4, True),
     ((12, 14, 16), 2, False), ((20, 9, 33), 2, True), ((7, 40, 12), 3, False)],
)
def test_adjoint_equals_oracle_adjoint(shape, nsweep, perturb):
    """Same derivative as the oracle's sequential reverse pass on every cell
    (the sums run in another order: 1e-12 of the largest entry). The
    perturb=False cases are pure layered models, where the slowness minima
    tie at almost every node."""
    src, rec = geometry(shape, 4, 30, 3)
    t_obs = oracle_times(velocity(shape, True, perturb=perturb), src, rec, nsweep)
    v0 = velocity(shape, False, perturb=perturb)
    T, g = gpu_gradient(v0, src, rec, nsweep, t_obs)
    # the forward is the reference's computation, bit for bit
    assert np.array_equal(T, oracle_times(v0, src, rec, nsweep))
    go = oracle_velocity_gradient(v0, src, rec, nsweep, t_obs)
    assert np.isfinite(g).all()
    assert np.abs(g - go).max() <= 1e-12 * np.abs(go).max()


def test_adjoint_matches_finite_differences_through_the_oracle():
    shape, nsweep = (12, 14, 16), 2
    src, rec = geometry(shape, 3, 24, 1)
    t_obs = oracle_times(velocity(shape, True), src, rec, nsweep)
    v0 = velocity(shape, False)
    _, g = gpu_gradient(v0, src, rec, nsweep, t_obs)
    gmax = np.abs(g).max()
    bad = []
    for c in check_cells(g):
        idx = np.unravel_index(c, shape)
        fd = central_difference(v0, idx, 1e-6, src, rec, nsweep, t_obs)
        if abs(fd - g[idx]) > 1e-6 * abs(fd) + 1e-10 * gmax:
            bad.append((idx, g[idx], fd))
    assert not bad, bad


def test_adjoint_is_deterministic_and_batched_equals_sum():
    shape, nsweep = (10, 12, 11), 4
    src, rec = geometry(shape, 4, 16, 2)
    v0 = velocity(shape, False)
    t_obs = oracle_times(velocity(shape, True), src, rec, nsweep)

    def grad(sel):
        return gpu_gradient(v0, src[sel], rec, nsweep, t_obs[sel])[1]

    g_all = grad(slice(None))
    assert np.array_equal(g_all, grad(slice(None)))  # run to run, bit for bit
    g_sum = sum(grad(slice(s, s + 1)) for s in range(len(src)))
    assert np.allclose(g_all, g_sum, rtol=1e-12, atol=1e-12 * np.abs(g_all).max())


def test_adjoint_with_zero_sweeps_and_outside_receivers():
    """nsweep=0 leaves only the source neighbourhood; receivers outside the
    grid contribute nothing (their traveltime is NaN and d/dT is zero)."""
    shape = (8, 9, 10)
    src, rec = geometry(shape, 2, 10, 4)
    rec = np.vstack([rec, [[-5.0, 3.0, 3.0]]])
    v0 = velocity(shape, False)
    for nsweep in (0, 1):
        vt = torch.tensor(v0, device="cuda", requires_grad=True)
        T = fp.traveltimes(vt, D, src, rec, nsweep)
        assert torch.isnan(T[:, -1]).all()
        r = torch.nan_to_num(T, nan=0.0)
        (0.5 * (r**2).sum()).backward()
        g = vt.grad.cpu().numpy()
        To = np.nan_to_num(oracle_times(v0, src, rec, nsweep))
        s = 1.0 / v0
        go = -O.adjoint3d(s, D, src, nsweep, rec, To) * s * s
        assert np.abs(g - go).max() <= 1e-12 * np.abs(go).max()


def test_reverse_pass_wait_timeout_is_reported_and_recoverable(monkeypatch):
    """The reverse pass's progress waits poll at most spin_limit times: with a
    limit of 1 it reports a timeout instead of hanging, and the next backward
    on the same context gives the exact gradient."""
    from fteikpy_gb300 import _adjoint

    shape, nsweep = (10, 12, 11), 2
    src, rec = geometry(shape, 3, 12, 6)
    v0 = velocity(shape, False)
    t_obs = oracle_times(velocity(shape, True), src, rec, nsweep)
    vt = torch.tensor(v0, device="cuda", requires_grad=True)
    T = fp.traveltimes(vt, D, src, rec, nsweep)
    loss = 0.5 * ((T - torch.as_tensor(t_obs, device="cuda")) ** 2).sum()
    monkeypatch.setattr(_adjoint, "SPIN_LIMIT", 1)
    with pytest.raises(RuntimeError, match="timed out"):
        loss.backward()
    monkeypatch.undo()
    _, g = gpu_gradient(v0, src, rec, nsweep, t_obs)
    go = oracle_velocity_gradient(v0, src, rec, nsweep, t_obs)
    assert np.abs(g - go).max() <= 1e-12 * np.abs(go).max()


@pytest.mark.parametrize("team", [0, 1])
def test_adjoint_through_either_sweep_kernel(team):
    """The taped forward runs in either sweep kernel (large batches use the
    team kernel): the gradient is the oracle adjoint's in both."""
    from fteikpy_gb300 import _lib

    lib = _lib.load()
    lib.fteik_set_option(b"sweep_team", team)
    try:
        shape, nsweep = (11, 13, 15), 2
        src, rec = geometry(shape, 6, 20, 8)
        t_obs = oracle_times(velocity(shape, True), src, rec, nsweep)
        v0 = velocity(shape, False)
        T, g = gpu_gradient(v0, src, rec, nsweep, t_obs)
        assert np.array_equal(T, oracle_times(v0, src, rec, nsweep))
        go = oracle_velocity_gradient(v0, src, rec, nsweep, t_obs)
        assert np.abs(g - go).max() <= 1e-12 * np.abs(go).max()
    finally:
        lib.fteik_set_option(b"sweep_team", -1)


def test_reverse_pass_chunk_does_not_change_the_gradient():
    """The reverse pass publishes its progress every `adjoint_chunk` steps;
    the schedule changes, the gradient's bits do not."""
    from fteikpy_gb300 import _lib

    lib = _lib.load()
    shape, nsweep = (13, 17, 22), 2
    src, rec = geometry(shape, 5, 25, 9)
    t_obs = oracle_times(velocity(shape, True), src, rec, nsweep)
    v0 = velocity(shape, False)
    grads = []
    try:
        for chunk in (1, 4, 64):
            assert lib.fteik_set_option(b"adjoint_chunk", chunk) == 0
            grads.append(gpu_gradient(v0, src, rec, nsweep, t_obs)[1])
    finally:
        lib.fteik_set_option(b"adjoint_chunk", -1)
    assert all(np.array_equal(grads[0], g) for g in grads[1:])
    go = oracle_velocity_gradient(v0, src, rec, nsweep, t_obs)
    assert np.abs(grads[0] - go).max() <= 1e-12 * np.abs(go).max()


def test_float32_velocity_and_a_single_receiver_are_converted():
    """A float32 velocity runs in float64 and gets its gradient back as
    float32; one receiver may be given as [3]. Both equal the float64 call."""
    shape, nsweep = (12, 14, 16), 2
    src, rec = geometry(shape, 2, 5, 3)
    v0 = velocity(shape, False, perturb=True).astype(np.float32).astype(np.float64)
    v32 = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    T32 = fp.traveltimes(v32, D, src, rec[0], nsweep)
    assert T32.shape == (len(src), 1) and T32.dtype == torch.float64
    T32.sum().backward()
    v64 = torch.tensor(v0, device="cuda", requires_grad=True)
    T64 = fp.traveltimes(v64, D, src, rec[:1], nsweep)
    T64.sum().backward()
    assert torch.equal(T32, T64)
    assert v32.grad.dtype == torch.float32
    assert torch.equal(v32.grad, v64.grad.to(torch.float32))


def test_source_chunks_and_recomputed_tapes_give_the_same_bits():
    """Sources split by a memory budget give the single-pass gradient bit for
    bit: the reverse pass in groups of sources over one solve's tape
    (fteik3d_adjoint_part), sources split into chunks (each with its own
    solve and tape, the gradient summed on in source order), and chunks whose
    tapes are dropped after the forward pass and solved again in the backward
    pass."""
    from fteikpy_gb300 import _adjoint, _lib

    lib = _lib.load()
    shape, nsweep = (12, 14, 16), 2
    src, rec = geometry(shape, 7, 20, 11)
    t_obs = oracle_times(velocity(shape, True), src, rec, nsweep)
    v0 = velocity(shape, False)
    T, g = gpu_gradient(v0, src, rec, nsweep, t_obs)
    need = _adjoint._chunk_plan(lib, shape, 7, nsweep, 1 << 50)[2]
    plans = []
    for budget in (need // 2, need // 3, 1):  # groups only; chunks and groups; all solved again
        plans.append(_adjoint._chunk_plan(lib, shape, 7, nsweep, budget)[:2])
        Tb, gb = gpu_gradient(v0, src, rec, nsweep, t_obs, memory_budget=budget)
        assert np.array_equal(Tb, T)
        assert np.array_equal(gb, g)
    assert plans[0][0] == 7 and plans[0][1] < 7
    assert plans[1][0] < 7 and plans[2] == (1, 1)
    go = oracle_velocity_gradient(v0, src, rec, nsweep, t_obs)
    assert np.abs(g - go).max() <= 1e-12 * np.abs(go).max()


def test_tape_overflow_is_reported_and_retried_with_more_history(monkeypatch):
    """Without history slots every repeated change of a node goes to the
    tape's overflow table, which then fills: the solve reports the overflow
    (no hang, no wrong tape). The autograd function retries with more slots
    and gets the same gradient; every slot count gives the same bits."""
    from fteikpy_gb300 import _adjoint, _device, _lib

    lib = _lib.load()
    shape, nsweep = (12, 14, 16), 2
    src, rec = geometry(shape, 7, 20, 12)
    t_obs = oracle_times(velocity(shape, True), src, rec, nsweep)
    v0 = velocity(shape, False)
    slow = _device.slowness(_device.to_device(v0))
    ws = torch.empty(lib.fteik3d_workspace_bytes(*shape, len(src), 2), dtype=torch.uint8,
                     device="cuda")
    with pytest.raises(RuntimeError, match="tape overflowed"):
        _adjoint._taped_solve(lib, slow, D, np.ascontiguousarray(src), nsweep, 0, ws)
    _, g = gpu_gradient(v0, src, rec, nsweep, t_obs)
    for steps in ([0, 6, 15], [1, 15], [15]):
        monkeypatch.setattr(_adjoint, "_history_steps", lambda n, s=steps: s)
        _, gh = gpu_gradient(v0, src, rec, nsweep, t_obs)
        assert np.array_equal(gh, g), steps
    monkeypatch.undo()
    go = oracle_velocity_gradient(v0, src, rec, nsweep, t_obs)
    assert np.abs(g - go).max() <= 1e-12 * np.abs(go).max()


def test_finite_differences_away_from_branch_ties_tomography_start_model():
    """The tomography workload on a reduced grid (24 x 32 x 32 cells, 16
    surface sources x 400 surface receivers, the linear-gradient start model
    and the anomaly's arrivals). On the exact start model every cell with a
    significant derivative enters a slowness minimum tied with a lateral
    neighbour (v depends on z only), where the solver has only one-sided
    derivatives; with the lateral ties broken (each cell within 0.1%), the
    gradient matches central differences (relative step 1e-6, through the
    oracle) to 1e-6 on 30 seeded cells away from every branch tie."""
    import bench

    shape = (24, 32, 32)
    v0, vt = bench.tomography_models(shape)
    src = bench.surface_sources(shape, n_side=4, seed=7)
    rec = bench.surface_receivers(shape, n=400, seed=11)
    t_obs = bench.oracle_receiver_times(O, vt, src, rec)[0]
    vb = bench.tie_broken(v0)
    _, g = gpu_gradient(vb, src, rec, 2, t_obs)
    res = bench.fd_check(O, vb, src, rec, t_obs, g, 30, True, 1e-2)
    assert res["cells"] == 30 and res["cells_within_1e-6"] == 30, res
    _, g0 = gpu_gradient(v0, src, rec, 2, t_obs)
    _, _, tied = bench.oracle_receiver_times(O, v0, src, rec, probe=True, margin=bench.TIE_MARGIN)
    pool = np.flatnonzero(np.abs(g0.ravel()) >= 1e-4 * np.abs(g0).max())
    assert len(pool) > 0 and not (~tied.ravel()[pool]).any()
