"""Slice-sharded Parareal host logic on CPU: one rank and two gloo ranks.

The propagators are small exact-arithmetic stand-ins written here (a linear
system y' = A y stepped by RK4 / forward Euler, in torch for the ranks and in
numpy for the oracle's serial replay of the reference's ``PararealOperator``),
so the test checks the slice partitioning, the correction exchange, the
replicated sweep, the termination rules and the trajectory gather.  Bar:
border points and trajectories within 1e-12 relative of the oracle; the
iteration count equal.
"""

import os
import socket

import numpy as np
import pytest

from oracle import fdm as ofdm
from pararealml_gb300.operators.parareal.sharded import SliceShardedParareal, slice_blocks

REL = 1e-12
V, C = 6, 2


def _matrix():
    rng = np.random.default_rng(3)
    a = rng.normal(0.0, 1.0, (V * C, V * C))
    return -(a @ a.T) / (V * C) - 0.2 * np.eye(V * C)


def _rk4_np(y, t0, t1, n=20):
    a = _matrix()
    h = (t1 - t0) / n
    y = y.reshape(-1).copy()
    for _ in range(n):
        k1 = a @ y
        k2 = a @ (y + 0.5 * h * k1)
        k3 = a @ (y + 0.5 * h * k2)
        k4 = a @ (y + h * k3)
        y = y + h / 6.0 * (k1 + 2 * k2 + 2 * k3 + k4)
    return y.reshape(V, C)


def _fe_np(y, t0, t1):
    return (y.reshape(-1) + (t1 - t0) * (_matrix() @ y.reshape(-1))).reshape(V, C)


def _rk4_traj_np(y, t0, t1, n=20):
    out = []
    h = (t1 - t0) / n
    for s in range(n):
        y = _rk4_np(y, t0 + s * h, t0 + (s + 1) * h, 1)
        out.append(y)
    return np.stack(out)


def _torch_props():
    import torch

    def fine(ys, ts, te):
        return torch.stack([torch.from_numpy(_rk4_np(y.numpy(), a, b)) for y, a, b in zip(ys, ts, te)])

    def coarse(y, a, b):
        return torch.from_numpy(_fe_np(y.numpy(), a, b))

    def traj(ys, ts, te):
        return torch.stack([torch.from_numpy(_rk4_traj_np(y.numpy(), a, b)) for y, a, b in zip(ys, ts, te)])

    return fine, coarse, traj


def _y0():
    return np.random.default_rng(8).normal(0.0, 1.0, (V, C))


def _oracle(S, tol, max_it, t=(0.0, 2.0)):
    return ofdm.parareal_solve(None, _y0(), t, S, _rk4_np, _fe_np, tol, max_it, fine_traj=_rk4_traj_np)


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _tc(kind):
    if kind == "scalar":
        return 1e-9
    if kind == "vector":
        return [1e-9, 1e-3]
    return lambda old, new: float(np.max(np.abs(new - old))) < 1e-7


def _solve(kind, S, max_it):
    import torch

    fine, coarse, traj = _torch_props()
    op = SliceShardedParareal(fine, coarse, _tc(kind), max_it, fine_trajectory=traj)
    return op.solve(torch.from_numpy(_y0()), (0.0, 2.0), S), op.last_stats


def test_slice_blocks_cover_the_slices_in_order():
    for S in range(1, 12):
        for world in range(1, S + 1):
            b = slice_blocks(S, world)
            assert b[0][0] == 0 and b[-1][1] == S
            assert all(b[k][1] == b[k + 1][0] for k in range(world - 1))
            sizes = [hi - lo for lo, hi in b]
            assert max(sizes) - min(sizes) <= 1 and min(sizes) >= 1
    with pytest.raises(ValueError):
        slice_blocks(2, 3)


@pytest.mark.parametrize("kind", ["scalar", "vector", "callable"])
def test_single_rank_matches_the_serial_replay(kind):
    S = 5
    out, stats = _solve(kind, S, 50)
    tol = _tc(kind)
    u, it, traj = _callable_oracle(S, tol) if callable(tol) else _oracle(S, tol, 50)
    assert out["iterations"] == it
    assert _rel(out["border_points"].numpy(), u) < REL
    assert _rel(out["trajectory"].numpy(), traj) < REL


def _callable_oracle(S, tc):
    """The oracle replay with a callable termination rule."""
    y0 = _y0()
    borders = np.linspace(0.0, 2.0, S + 1)
    g = []
    y = y0
    for j in range(S):
        y = _fe_np(y, borders[j], borders[j + 1])
        g.append(y)
    g = np.stack(g)
    u = np.concatenate([y0[None], g])
    start = None
    it = 0
    for i in range(S):
        start = u.copy()
        corr = np.stack([_rk4_np(u[j], borders[j], borders[j + 1]) for j in range(S)]) - g
        old = u[1:].copy()
        for j in range(i, S):
            if j > i:
                g[j] = _fe_np(u[j], borders[j], borders[j + 1])
            u[j + 1] = g[j] + corr[j]
        it = i + 1
        if tc(old, u[1:]):
            break
    parts = []
    for j in range(S):
        sub = _rk4_traj_np(start[j], borders[j], borders[j + 1])
        parts.append(sub + (u[j + 1] - sub[-1]))
    return u, it, np.concatenate(parts)


def test_max_iterations_caps_the_loop():
    out, _ = _solve("scalar", 6, 2)
    u, it, traj = _oracle(6, 1e-9, 2)
    assert out["iterations"] == it == 2
    assert _rel(out["border_points"].numpy(), u) < REL


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir, kind, S, max_it):
    import torch
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        out, stats = _solve(kind, S, max_it)
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), u=out["border_points"].numpy(),
                 traj=out["trajectory"].numpy(), it=out["iterations"], lo=stats["slices"][0], hi=stats["slices"][1])
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("kind,S,max_it", [("scalar", 5, 50), ("callable", 4, 50), ("vector", 7, 3)])
def test_two_gloo_ranks_match_the_serial_replay(tmp_path, kind, S, max_it):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path), kind, S, max_it), nprocs=world,
                       join=True, start_method="spawn")
    tc = _tc(kind)
    u, it, traj = _callable_oracle(S, tc) if callable(tc) else _oracle(S, tc, max_it)
    blocks = slice_blocks(S, world)
    for r in range(world):
        res = np.load(tmp_path / f"rank{r}.npz")
        assert (int(res["lo"]), int(res["hi"])) == blocks[r]
        assert int(res["it"]) == it
        assert _rel(res["u"], u) < REL
        assert _rel(res["traj"], traj) < REL


def _failing_rank_main(rank, world, port, outdir):
    """Rank 1's fine propagator raises in the second iteration; rank 0 must
    leave its next collective with an error instead of waiting forever."""
    import datetime
    import time

    import torch
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=10))
    fine, coarse, _ = _torch_props()
    calls = [0]

    def flaky_fine(ys, ts, te):
        calls[0] += 1
        if rank == 1 and calls[0] == 2:
            raise RuntimeError("injected failure on rank 1")
        return fine(ys, ts, te)

    op = SliceShardedParareal(flaky_fine, coarse, 1e-12, 50)
    t0 = time.time()
    try:
        op.solve(torch.from_numpy(_y0()), (0.0, 2.0), 6)
        outcome = "finished"
    except Exception as e:  # the failure under test
        outcome = type(e).__name__
    with open(os.path.join(outdir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{outcome} {time.time() - t0:.2f}")
    if rank == 1:
        # leave between collectives: closing this rank's connections is what
        # the other rank sees
        dist.destroy_process_group()
    else:
        try:
            dist.destroy_process_group()
        except Exception:  # the peer is gone
            pass


def test_a_failing_gloo_rank_ends_the_other_ranks_collective(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_failing_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    r1 = (tmp_path / "rank1.txt").read_text().split()
    r0 = (tmp_path / "rank0.txt").read_text().split()
    assert r1[0] == "RuntimeError"
    assert r0[0] != "finished"  # the collective of the surviving rank failed
    assert float(r0[1]) < 60.0


def test_whole_interval_first_prediction():
    """The reference's first coarse prediction is one coarse solve over the
    whole interval sampled at the slice ends; given that callable the
    runner uses it, with the same iterates as the chained prediction for
    this time-independent system."""
    import torch

    fine, coarse, traj = _torch_props()
    S = 5
    borders = np.linspace(0.0, 2.0, S + 1)

    def whole(y0, t0, t1, n):
        ends, y = [], y0
        for j in range(n):
            y = coarse(y, borders[j], borders[j + 1])
            ends.append(y)
        whole.calls += 1
        return torch.stack(ends)

    whole.calls = 0
    op = SliceShardedParareal(fine, coarse, 1e-9, 50, fine_trajectory=traj, coarse_whole=whole)
    out = op.solve(torch.from_numpy(_y0()), (0.0, 2.0), S)
    u, it, _ = _oracle(S, 1e-9, 50)
    assert whole.calls == 1
    assert out["iterations"] == it
    assert _rel(out["border_points"].numpy(), u) < REL
