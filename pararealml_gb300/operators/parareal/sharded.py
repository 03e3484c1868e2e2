"""Parareal with its time slices split across ranks (one process per GPU).

Reference: ``pararealml/operators/parareal/parareal_operator.py:102-197``
runs one MPI rank per time slice.  Each iteration the ranks run the fine
operator on their own slice, ``comm.Allgather`` the corrections (``:165``)
and replay the sequential coarse sweep redundantly.  When the iteration ends,
they gather the shifted fine trajectories with a second ``Allgather``
(``:193``).

Here a rank owns a contiguous block of slices (block sizes differ by at most
one when the slice count does not divide).  It runs the fine propagator on the
open slices of its block (``j >= i`` in iteration ``i``) as ONE batch, and the
corrections of all blocks are exchanged by one ``all_gather`` per iteration
(NCCL between GPUs, gloo between CPU processes; blocks are zero-padded to the
largest block for the collective).  The coarse sweep, the update norms and
the termination test are replicated: every rank holds bit-identical border
points and so reaches the same decision without another exchange.  The
optional fine trajectory is gathered once at the end, like the reference's
second ``Allgather``.

States are float64 tensors of any shape whose last axis is the component
axis (the reference's ``(*vertices, C)``), on the device the propagators
use.  ``FDMSlicePropagator`` wraps an ``FDMOperator`` plan as such a
propagator on the GPU.
"""

from __future__ import annotations

import sys
from typing import Callable, List, Optional, Sequence, Tuple, Union

import numpy as np


def slice_blocks(n_slices: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous ``[lo, hi)`` slice ranges of the ranks, sizes differing by at most one."""
    if n_slices < 1 or world < 1:
        raise ValueError("slice and rank counts must be at least 1")
    if world > n_slices:
        raise ValueError(f"{world} ranks for {n_slices} slices: every rank needs at least one slice")
    base, extra = divmod(n_slices, world)
    out, lo = [], 0
    for r in range(world):
        hi = lo + base + (1 if r < extra else 0)
        out.append((lo, hi))
        lo = hi
    return out


def rms_update_norms(old, new):
    """Per component, the largest over slices of the RMS change of a border
    point (``parareal_operator.py:85-100``); ``old``/``new``: (S, *V, C)."""
    import torch

    d = (new - old).reshape(new.shape[0], -1, new.shape[-1])
    return torch.sqrt((d * d).mean(dim=1)).amax(dim=0)


class SliceShardedParareal:
    """Slice-sharded Parareal over ``torch.distributed`` ranks.

    ``fine(ys, t_starts, t_ends)`` propagates a batch ``ys`` (k, *shape) of
    slice start states to the slice ends; ``coarse(y, t_start, t_end)`` does
    the same for one state.  ``termination_condition`` is the reference's:
    one tolerance, one per component, or a callable on the previous and new
    border points as numpy arrays (``parareal_operator.py:53-100``).
    ``fine_trajectory(ys, t_starts, t_ends)`` (optional) returns every fine
    step of a batch of slices, (k, n_steps, *shape).  ``coarse_whole(y0,
    t_start, t_end, n_slices)`` (optional) returns the slice-end states
    (n_slices, *shape) of ONE coarse solve over the whole interval, the
    reference's first prediction (``parareal_operator.py:131-137``: one
    ``g.solve(ivp)`` sampled at the slice ends); without it the first
    prediction chains one coarse call per slice.
    """

    def __init__(
        self,
        fine: Callable,
        coarse: Callable,
        termination_condition: Union[float, Sequence[float], Callable[[np.ndarray, np.ndarray], bool]],
        max_iterations: int = sys.maxsize,
        group=None,
        fine_trajectory: Optional[Callable] = None,
        coarse_whole: Optional[Callable] = None,
    ):
        if max_iterations < 1:
            raise ValueError("max_iterations must be at least 1")
        self._fine = fine
        self._coarse = coarse
        self._tc = termination_condition
        self._max_iterations = max_iterations
        self._group = group
        self._fine_trajectory = fine_trajectory
        self._coarse_whole = coarse_whole
        self.last_stats: dict = {}

    def _ranks(self) -> Tuple[int, int]:
        import torch.distributed as dist

        if dist.is_available() and dist.is_initialized():
            return dist.get_rank(self._group), dist.get_world_size(self._group)
        return 0, 1

    def _all_gather(self, local, blocks):
        """Concatenates every rank's block (``local`` is padded to the widest block)."""
        import torch
        import torch.distributed as dist

        if len(blocks) == 1:
            return local[: blocks[0][1] - blocks[0][0]]
        parts = [torch.empty_like(local) for _ in blocks]
        dist.all_gather(parts, local.contiguous(), group=self._group)
        return torch.cat([p[: hi - lo] for p, (lo, hi) in zip(parts, blocks)])

    def _tolerances(self, n_comp: int) -> Optional[np.ndarray]:
        if callable(self._tc):
            return None
        if isinstance(self._tc, (int, float)):
            return np.full(n_comp, float(self._tc))
        tol = np.asarray(self._tc, dtype=np.float64)
        if tol.shape != (n_comp,):
            raise ValueError(f"termination condition needs {n_comp} tolerances, got {tol.shape}")
        return tol

    def solve(self, y0, t_interval, n_slices: int) -> dict:
        """Parareal from ``y0`` (float64 tensor (*V, C)) over ``t_interval``.

        Returns ``{"border_points": U (S+1, *V, C), "iterations": n,
        "norm_history": [...], "trajectory": (S * steps, *V, C) or None}``,
        identical on every rank.
        """
        import torch

        rank, world = self._ranks()
        S = int(n_slices)
        blocks = slice_blocks(S, world)
        lo, hi = blocks[rank]
        width = max(h - l for l, h in blocks)
        t0, t1 = float(t_interval[0]), float(t_interval[1])
        borders = np.linspace(t0, t1, S + 1)
        tol = self._tolerances(y0.shape[-1])

        U = torch.empty((S + 1,) + tuple(y0.shape), dtype=torch.float64, device=y0.device)
        G = torch.empty((S,) + tuple(y0.shape), dtype=torch.float64, device=y0.device)
        U[0] = y0
        if self._coarse_whole is not None:
            G[:] = self._coarse_whole(y0, t0, t1, S)
            U[1:] = G
        else:
            for j in range(S):
                G[j] = self._coarse(U[j], borders[j], borders[j + 1])
                U[j + 1] = G[j]

        history: List[np.ndarray] = []
        iterations = 0
        U_start = None
        for i in range(min(S, self._max_iterations)):
            U_start = U[:-1].clone()
            corr_local = torch.zeros((width,) + tuple(y0.shape), dtype=torch.float64, device=y0.device)
            first = max(lo, i)
            if first < hi:
                fe = self._fine(U[first:hi], borders[first:hi], borders[first + 1 : hi + 1])
                corr_local[first - lo : hi - lo] = fe - G[first:hi]
            corr = self._all_gather(corr_local, blocks)
            old = U[1:].clone()
            for j in range(i, S):
                if j > i:
                    G[j] = self._coarse(U[j], borders[j], borders[j + 1])
                U[j + 1] = G[j] + corr[j]
            iterations = i + 1
            if tol is None:
                stop = bool(self._tc(old.cpu().numpy(), U[1:].cpu().numpy()))
            else:
                nrm = rms_update_norms(old, U[1:]).cpu().numpy()
                history.append(nrm)
                stop = bool(np.all(nrm < tol))
            if stop:
                break

        trajectory = None
        if self._fine_trajectory is not None:
            sub = self._fine_trajectory(U_start[lo:hi], borders[lo:hi], borders[lo + 1 : hi + 1])
            sub = sub + (U[lo + 1 : hi + 1] - sub[:, -1]).unsqueeze(1)
            pad = torch.zeros((width,) + tuple(sub.shape[1:]), dtype=sub.dtype, device=sub.device)
            pad[: hi - lo] = sub
            trajectory = self._all_gather(pad, blocks).reshape((-1,) + tuple(y0.shape))
        self.last_stats = {"iterations": iterations, "norm_history": [h.tolist() for h in history],
                           "slices": (lo, hi), "world": world}
        return {"border_points": U, "iterations": iterations, "norm_history": history, "trajectory": trajectory}


class FDMSlicePropagator:
    """Propagates batches of float64 channel-last device states over one time
    slice with an ``FDMOperator`` (fused stencil kernel, one batched run)."""

    def __init__(self, op, cp, max_batch: int, delta_t: float, trajectory: bool = False):
        import torch

        self.cp = cp
        n = int(round(delta_t / op.d_t))
        if n < 1 or not np.isclose(n * op.d_t, delta_t):
            raise ValueError(f"d_t {op.d_t} does not divide the slice length {delta_t}")
        self.op, self.n_steps = op, n
        self.plan = op.plan(cp, max_batch)
        self.max_batch = max_batch
        self.state = self.plan.new_state(1)[0]
        self.trajectory = trajectory
        self.out = self.plan.new_state(n if trajectory else 1)
        self.work = self.plan.new_state(2) if (n > 1 and not trajectory) else None
        self.t_off = torch.zeros(max_batch, dtype=torch.float64, device=self.plan.device)

    def _run(self, ys, t_starts):
        import torch

        single = ys.dim() == len(self.plan.low.vertices_shape) + 1
        if single:
            ys = ys.unsqueeze(0)
            t_starts = [t_starts]
        k = ys.shape[0]
        if k > self.max_batch:
            raise ValueError(f"batch {k} above the propagator's {self.max_batch}")
        self.plan.pack_device(ys.contiguous(), self.state[:k])
        self.t_off[:k] = torch.as_tensor(np.asarray(t_starts, dtype=np.float64).reshape(-1), device=self.t_off.device)
        if self.trajectory:
            self.plan.run(self.state, self.out, self.n_steps, 0.0, self.op.d_t, save_every=1, batch=k,
                          traj_step_stride=self.plan.batch * self.plan.inst, t_offset_ptr=self.t_off.data_ptr())
        else:
            self.plan.run(self.state, self.out[0], self.n_steps, 0.0, self.op.d_t, save_every=self.n_steps,
                          work=self.work, batch=k, t_offset_ptr=self.t_off.data_ptr())
        return single, k

    def __call__(self, ys, t_starts, t_ends=None):
        single, k = self._run(ys, t_starts)
        out = self.plan.unpack(self.out[-1] if self.trajectory else self.out[0], k)
        return out[0] if single else out

    def steps(self, ys, t_starts, t_ends=None):
        """Every fine step of each slice: (k, n_steps, *V, C)."""
        import torch

        if not self.trajectory:
            raise ValueError("built without trajectory storage")
        _, k = self._run(ys, t_starts)
        return torch.stack([self.plan.unpack(self.out[s], k) for s in range(self.n_steps)], dim=1)

    def whole(self, y0, t_start: float, t_end: float, n_slices: int):
        """Slice-end states (n_slices, *V, C) of ONE solve of ``y0`` from
        ``t_start`` over n_slices slice lengths (the reference's first
        coarse prediction, a single ``g.solve(ivp)``)."""
        plan = self.op.plan(self.cp, 1)
        s0 = plan.new_state(1)
        plan.pack_device(y0.unsqueeze(0).contiguous(), s0[0])
        ends = plan.new_state(n_slices)
        work = plan.new_state(2) if self.n_steps > 1 else None
        plan.run(s0[0], ends, self.n_steps * n_slices, float(t_start), self.op.d_t, save_every=self.n_steps, work=work)
        return plan.unpack(ends, n_slices)
