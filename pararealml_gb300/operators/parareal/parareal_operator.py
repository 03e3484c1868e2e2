"""Single-GPU batched Parareal with the reference's ``PararealOperator`` surface.

Reference: ``pararealml/operators/parareal/parareal_operator.py:13-197``.
There, every MPI rank owns one time slice: each iteration the ranks run the
fine operator on their slice in parallel, allgather the corrections
``F(U_j) - G_old(U_j)`` and replay the sequential coarse sweep
``U_{j+1} = G(U_j) + correction_j`` redundantly, until the largest per-slice
RMS update of every component is below the tolerance.

Here the time slices (``n_slices``, the reference's ``comm.size``) and any
number of initial value problems sharing one constrained problem are batch
dimensions of device arrays on one GPU:

* the fine sweep is ONE batched run of the fused stencil kernel over
  slices x instances (slices already converged, j < i, are skipped: their
  fine results cannot change any more);
* the border points U, the coarse end points, the corrections, the update
  norms and the termination test are FP64 and stay on the device
  (``csrc/prml_parareal.cu``); only the per-instance norms cross to the host;
* the coarse sweep is a chain of launches on one stream;
* each instance terminates on its own, exactly as the reference's loop for
  that problem would (border points of finished instances are frozen).

Solutions are the reference's: the fine trajectory of the last iteration,
each slice shifted by the constant ``U_{j+1} - F_end_j`` (``:192``).
"""

from __future__ import annotations

import sys
from typing import Callable, List, Optional, Sequence, Union

import numpy as np

from ... import _native
from ...operator import Operator, discretize_time_domain
from ...solution import Solution
from ..fdm.fdm_operator import FDMOperator


class FDMCoarsePropagator:
    """Coarse propagation of a batch of device states by an ``FDMOperator``."""

    def __init__(self, op: FDMOperator, cp, batch: int, n_steps: int):
        self.op = op
        self.plan = op.plan(cp, batch)
        self.n_steps = n_steps
        self.work = self.plan.new_state(2) if n_steps > 1 else None
        self.dtype = op.dtype

    def __call__(self, src, dst, t_start: float) -> None:
        self.plan.run(src, dst, self.n_steps, t_start, self.op.d_t, save_every=self.n_steps, work=self.work)


class PararealOperator(Operator):
    def __init__(
        self,
        f: Operator,
        g: Operator,
        termination_condition: Union[float, Sequence[float], Callable[[np.ndarray, np.ndarray], bool]] = None,
        max_iterations: int = sys.maxsize,
        *,
        n_slices: int = 1,
        trajectory: Union[str, int] = "full",
        keep_on_device: bool = False,
    ):
        super().__init__(f.d_t, f.vertex_oriented)
        if not isinstance(f, FDMOperator):
            raise NotImplementedError("the fine operator must be a GPU FDMOperator")
        if n_slices < 1:
            raise ValueError("n_slices must be at least 1")
        if not (trajectory in ("full", "final") or (isinstance(trajectory, int) and trajectory >= 1)):
            raise ValueError("trajectory must be 'full', 'final' or a positive int stride")
        self._f = f
        self._g = g
        self._termination_condition = termination_condition
        self._max_iterations = max_iterations
        self._n_slices = n_slices
        self._trajectory = trajectory
        self._keep_on_device = keep_on_device
        self.last_stats: dict = {}

    # ------------------------------------------------------------------
    def solve(self, ivp, parallel_enabled: bool = True) -> Solution:
        if not parallel_enabled:
            return self._f.solve(ivp)
        return self.solve_batch([ivp])[0]

    def solve_batch(self, ivps: Sequence) -> List[Solution]:
        """Solves several IVPs that share one constrained problem and time
        interval as one batched Parareal run."""
        if not ivps:
            return []
        cp = ivps[0].constrained_problem
        t_interval = tuple(ivps[0].t_interval)
        for ivp in ivps[1:]:
            if ivp.constrained_problem is not cp or tuple(ivp.t_interval) != t_interval:
                raise ValueError("batched IVPs must share the constrained problem and time interval")
        y0 = np.stack([np.asarray(ivp.initial_condition.discrete_y_0(self._vertex_oriented), dtype=np.float64) for ivp in ivps])
        result = self.run(cp, y0, t_interval)
        sols = []
        for b, ivp in enumerate(ivps):
            y = result["trajectory"][b] if result["trajectory"] is not None else result["final"][b][np.newaxis]
            t = result["t"]
            d_t = result["d_t"]
            if self._keep_on_device:
                sols.append(Solution(ivp, t, y, vertex_oriented=self._vertex_oriented, d_t=d_t))
            else:
                sols.append(Solution(ivp, t, y.cpu().numpy(), vertex_oriented=self._vertex_oriented, d_t=d_t))
        return sols

    # ------------------------------------------------------------------
    def _check_step(self, op, delta_t, which):
        if not np.isclose(delta_t, op.d_t * round(delta_t / op.d_t)):
            raise ValueError(
                f"{which} operator time step size ({op.d_t}) must be a "
                f"divisor of sub-IVP time slice length ({delta_t})"
            )

    def _tolerances(self, n_comp: int) -> Optional[np.ndarray]:
        tc = self._termination_condition
        if callable(tc):
            return None
        if isinstance(tc, Sequence) and not isinstance(tc, str):
            if len(tc) != n_comp:
                raise ValueError(
                    f"length of update tolerances ({len(tc)}) must match number of y dimensions ({n_comp})"
                )
            return np.array(tc, dtype=np.float64)
        return np.array([tc] * n_comp, dtype=np.float64)

    def _coarse(self, cp, batch: int, n_steps: int):
        g = self._g
        if isinstance(g, FDMOperator):
            return FDMCoarsePropagator(g, cp, batch, n_steps)
        make = getattr(g, "coarse_propagator", None)
        if make is None:
            raise NotImplementedError("the coarse operator must be a GPU FDMOperator or provide coarse_propagator()")
        return make(cp, batch, n_steps)

    def run(self, cp, y0: np.ndarray, t_interval):
        """Batched Parareal on device.

        ``y0``: float64 (batch, *vertices, C).  Returns a dict with the
        device float64 final states, the trajectory (or None), its time
        points, per-instance iteration counts and the update-norm history.
        """
        import torch

        S = self._n_slices
        B = y0.shape[0]
        t0, t1 = float(t_interval[0]), float(t_interval[1])
        delta_t = (t1 - t0) / S
        self._check_step(self._f, delta_t, "fine")
        self._check_step(self._g, delta_t, "coarse")
        if self._max_iterations < 1:
            raise ValueError("max_iterations must be at least 1")
        n_f = int(round(delta_t / self._f.d_t))
        n_g = int(round(delta_t / self._g.d_t))
        borders = np.linspace(t0, t1, S + 1)
        C = cp.differential_equation.y_dimension
        tol = self._tolerances(C)
        lib = _native.lib()
        stream = torch.cuda.current_stream().cuda_stream

        fplan = self._f.plan(cp, S * B)
        coarse = self._coarse(cp, B, n_g)
        dev = fplan.device
        inst = fplan.inst
        shape = (B, C, fplan.nx, fplan.pitch)
        f64 = torch.float64
        ftype = {"f32": torch.float32, "f64": torch.float64}[fplan.dtype]
        gtype = {"f32": torch.float32, "f64": torch.float64}[coarse.dtype]
        fes = fplan.esize
        ges = 4 if coarse.dtype == "f32" else 8

        U = torch.empty((S + 1,) + shape, dtype=f64, device=dev)
        U_start = torch.empty_like(U)
        g_old = torch.empty((S,) + shape, dtype=f64, device=dev)
        corr = torch.zeros((S,) + shape, dtype=f64, device=dev)
        old = torch.empty((S,) + shape, dtype=f64, device=dev)
        f_in = torch.empty((S,) + shape, dtype=ftype, device=dev)
        f_end = torch.empty((S,) + shape, dtype=ftype, device=dev)
        f_work = torch.empty((2, S) + shape, dtype=ftype, device=dev) if n_f > 1 else None
        g_in = torch.empty(shape, dtype=gtype, device=dev)
        g_out = torch.empty(shape, dtype=gtype, device=dev)
        t_offsets = torch.tensor(np.repeat(borders[:-1], B), dtype=f64, device=dev)
        active = torch.ones(B, dtype=torch.int32, device=dev)
        chunks = max(1, min(64, (fplan.nx * fplan.ny) // 4096))
        partial = torch.empty(lib.prml_pr_norm_scratch_elems(S, B, C, chunks), dtype=f64, device=dev)
        norms = torch.empty((B, C), dtype=f64, device=dev)
        n_slice = B * inst  # elements per slice block

        y0_dev = torch.from_numpy(np.ascontiguousarray(y0)).to(dev)
        fplan.pack_device(y0_dev, U[0], esize=8)

        def ptr(t, j=0, es=8):
            return t.data_ptr() + j * n_slice * es

        chk = _native.check
        # initial coarse pass: U_{j+1} = G(U_j) (corrections are zero)
        chk(lib.prml_pr_cast(ptr(U, 0), g_in.data_ptr(), ges, n_slice, stream), "cast")
        for j in range(S):
            coarse(g_in, g_out, float(borders[j]))
            chk(lib.prml_pr_advance(g_out.data_ptr(), ges, ptr(g_old, j), ptr(corr, j), ptr(U, j + 1),
                                    g_in.data_ptr(), n_slice, inst, None, B, stream), "advance")

        iterations = np.zeros(B, dtype=np.int64)
        done = np.zeros(B, dtype=bool)
        history = []
        for i in range(min(S, self._max_iterations)):
            act = active.data_ptr()
            # border points at the start of this iteration, per live instance
            chk(lib.prml_pr_copy(ptr(U, 0), ptr(U_start, 0), (S + 1) * n_slice, inst, act, B, stream), "copy")
            # fine sweep over the slices that can still change (j >= i), batched
            m = S - i
            chk(lib.prml_pr_cast(ptr(U, i), ptr(f_in, i, fes), fes, m * n_slice, stream), "cast")
            fplan.run(
                ptr(f_in, i, fes), ptr(f_end, i, fes), n_f, 0.0, self._f.d_t, save_every=n_f,
                work=(ptr(f_work[0], i, fes), ptr(f_work[1], i, fes)) if f_work is not None else None,
                batch=m * B, t_offset_ptr=t_offsets.data_ptr() + i * B * 8,
            )
            chk(lib.prml_pr_correct(ptr(f_end, i, fes), fes, ptr(g_old, i), ptr(corr, i), m * n_slice,
                                    inst, act, B, stream), "correct")
            chk(lib.prml_pr_copy(ptr(U, 1), ptr(old, 0), S * n_slice, inst, None, B, stream), "copy")
            # coarse sweep
            chk(lib.prml_pr_advance(None, ges, ptr(g_old, i), ptr(corr, i), ptr(U, i + 1),
                                    g_in.data_ptr(), n_slice, inst, act, B, stream), "advance")
            for j in range(i + 1, S):
                coarse(g_in, g_out, float(borders[j]))
                chk(lib.prml_pr_advance(g_out.data_ptr(), ges, ptr(g_old, j), ptr(corr, j), ptr(U, j + 1),
                                        g_in.data_ptr(), n_slice, inst, act, B, stream), "advance")
            iterations[~done] = i + 1
            if tol is not None:
                chk(lib.prml_pr_update_norm(ptr(U, 1), ptr(old, 0), S, B, C, fplan.nx, fplan.ny, fplan.pitch,
                                            chunks, partial.data_ptr(), norms.data_ptr(), stream), "norm")
                nrm = norms.cpu().numpy()
                history.append(nrm.copy())
                finished = np.all(nrm < tol[np.newaxis, :], axis=1)
            else:
                finished = np.array([self._callable_check(fplan, U, old, b, S) for b in range(B)])
            newly = finished & ~done
            if newly.any():
                done |= newly
                active.copy_(torch.from_numpy((~done).astype(np.int32)))
            if done.all():
                break

        fplan.check_status()
        final = fplan.unpack(U[S], B, esize=8)
        out = {
            "final": final,
            "trajectory": None,
            "t": np.array([t1]),
            "d_t": t1 - t0,
            "iterations": iterations,
            "norm_history": history,
            "border_points": U,
        }
        if self._trajectory != "final":
            out.update(self._fine_trajectory(fplan, U, U_start, f_in, S, B, n_f, t_interval, t_offsets, fes))
        self.last_stats = {"iterations": iterations.tolist(), "norm_history": [h.tolist() for h in history]}
        return out

    def _callable_check(self, fplan, U, old, b, S) -> bool:
        new = fplan.unpack(U[1:, b], S, esize=8).cpu().numpy()
        prev = fplan.unpack(old[:, b], S, esize=8).cpu().numpy()
        return bool(self._termination_condition(prev, new))

    def _fine_trajectory(self, fplan, U, U_start, f_in, S, B, n_f, t_interval, t_offsets, fes):
        """The last iteration's fine sub-trajectories, each shifted so that it
        ends on the corrected border point (parareal_operator.py:190-193)."""
        import torch

        lib = _native.lib()
        stream = torch.cuda.current_stream().cuda_stream
        every = 1 if self._trajectory == "full" else int(self._trajectory)
        if n_f % every:
            raise ValueError(f"trajectory stride {every} must divide the fine steps per slice ({n_f})")
        n_save = n_f // every
        inst = fplan.inst
        n_slice = B * inst
        _native.check(lib.prml_pr_cast(U_start.data_ptr(), f_in.data_ptr(), fes, S * n_slice, stream), "cast")
        traj = fplan.new_state(n_save)  # (n_save, S*B, C, nx, pitch)
        fplan.run(f_in, traj, n_f, 0.0, self._f.d_t, save_every=every, t_offset_ptr=t_offsets.data_ptr())
        delta = torch.empty((S * B,) + tuple(traj.shape[2:]), dtype=torch.float64, device=traj.device)
        _native.check(
            lib.prml_pr_end_delta(U[1:].data_ptr(), traj[n_save - 1].data_ptr(), fes, delta.data_ptr(), S * n_slice, stream),
            "end delta",
        )
        y = fplan.unpack(traj, n_save * S * B)  # (n_save*S*B, *V, C) float64
        vshape = tuple(y.shape[1:])
        y = y.view((n_save, S, B) + vshape)
        shift = fplan.unpack(delta, S * B, esize=8).view((S, B) + vshape)
        y = y + shift.unsqueeze(0)
        y = y.permute(2, 1, 0, *range(3, 3 + len(vshape))).reshape((B, S * n_save) + vshape)
        t = discretize_time_domain(t_interval, self._f.d_t)[1:]
        t = t[every - 1:: every]
        return {"trajectory": y, "t": t, "d_t": self._f.d_t * every}
