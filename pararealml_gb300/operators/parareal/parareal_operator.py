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
  that problem would (border points of finished instances are frozen);
* time-dependent boundary conditions: the fine and coarse plans hold one
  set of half-step boundary tables over the whole interval and every slice
  reads it from its own start time (per-instance table offsets), as each
  rank's sub-IVP in the reference evaluates its conditions on its slice;
* implicit operators (backward Euler, Crank-Nicolson): the fine sweep runs
  one secant-driven run per open slice at its own start time, and the work
  units run eagerly (their iterations stop on counters the host reads).

Solutions are the reference's: the fine trajectory of the last iteration,
each slice shifted by the constant ``U_{j+1} - F_end_j`` (``:192``).
"""

from __future__ import annotations

import sys
from typing import Callable, List, Optional, Sequence, Union

import numpy as np

from ... import _native
from ...engine import to_host
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
        fallback: Optional[Operator] = None,
        use_graphs: bool = True,
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
        self._fallback = fallback
        self._use_graphs = use_graphs
        self._ws = None
        self._last_delta_t = None
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
                sols.append(Solution(ivp, t, to_host(y), vertex_oriented=self._vertex_oriented, d_t=d_t,
                                     copy=False))
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
        return self._make_coarse(self._g, cp, batch, n_steps)

    def _make_coarse(self, g, cp, batch: int, n_steps: Optional[int] = None):
        if n_steps is None:
            n_steps = int(round((self._last_delta_t) / g.d_t))
        if isinstance(g, FDMOperator):
            return FDMCoarsePropagator(g, cp, batch, n_steps)
        make = getattr(g, "coarse_propagator", None)
        if make is None:
            raise NotImplementedError("the coarse operator must be a GPU FDMOperator or provide coarse_propagator()")
        return make(cp, batch, n_steps)

    def run(self, cp, y0: np.ndarray, t_interval, monitor: Optional[Callable] = None):
        """Batched Parareal on device.

        ``y0``: float64 (batch, *vertices, C), a host array or a CUDA
        tensor.  Returns a dict with the
        device float64 final states, the trajectory (or None), its time
        points, per-instance iteration counts and the update-norm history.

        ``monitor(i, final_border)`` (optional) is called on the host after
        iteration i (0-based) has been issued and its termination test has
        run, with the device float64 border point at the interval's end
        (batch, C, rows, pitch; the planar layout, overwritten by the next
        iteration): a caller that measures error against iterations copies
        it or records an event there.
        """
        import torch

        from ..fdm.fdm_operator import _initial_state

        if cp.differential_equation.x_dimension and not cp.are_all_boundary_conditions_static:
            # the reference's whole-interval coarse solve and first fine slice
            # constrain the initial state at t0 (fdm_operator.py:56-63); every
            # later border point already satisfies the Dirichlet values at its
            # time (sums and differences of constrained solver outputs)
            y0 = np.stack([_initial_state(cp, float(t_interval[0]), y)
                           for y in (y0.cpu().numpy() if hasattr(y0, "cpu") else np.asarray(y0))])
        if any(int(getattr(k, "value", k)) == 2 for k in cp.differential_equation.symbolic_equation_system.lhs_types):
            raise NotImplementedError(
                "LHS.Y_LAPLACIAN: each Jacobi solve starts from a random estimate drawn per MPI rank in "
                "the reference, an order a batched run over all slices cannot reproduce"
            )
        S = self._n_slices
        B = y0.shape[0]
        t0, t1 = float(t_interval[0]), float(t_interval[1])
        delta_t = (t1 - t0) / S
        self._check_step(self._f, delta_t, "fine")
        self._check_step(self._g, delta_t, "coarse")
        if self._fallback is not None:
            self._check_step(self._fallback, delta_t, "fallback coarse")
        self._last_delta_t = delta_t
        if self._max_iterations < 1:
            raise ValueError("max_iterations must be at least 1")
        C = cp.differential_equation.y_dimension
        tol = self._tolerances(C)
        _native.lib()

        key = (id(cp), B, t0, t1, S)
        ws = self._ws if (self._ws is not None and self._ws.key == key and self._ws.cp is cp) else None
        if ws is None:
            ws = _Workspace(self, cp, B, t0, t1, key)
            self._ws = ws
        ws.pack_y0(y0)
        ws.reset()
        g = ws.coarse("g")
        ws.run_unit(("init", "g"), lambda: ws.init_sweep(g))

        iterations = np.zeros(B, dtype=np.int64)
        done = np.zeros(B, dtype=bool)
        history = []
        fallback_at = None
        gname = "g"
        for i in range(min(S, self._max_iterations)):
            ws.run_unit(("iter", i, gname, tol is not None), lambda i=i, g=g: ws.iteration(i, g, tol is not None))
            iterations[~done] = i + 1
            if tol is not None:
                nrm = ws.norms.cpu().numpy()
                history.append(nrm.copy())
                finished = np.all(nrm < tol[np.newaxis, :], axis=1)
            else:
                finished = np.array([self._callable_check(ws.fplan, ws.U, ws.old, b, S) for b in range(B)])
            newly = finished & ~done
            if newly.any():
                done |= newly
                ws.active.copy_(torch.from_numpy((~done).astype(np.int32)))
            if monitor is not None:
                monitor(i, ws.U[S])
            if done.all():
                break
            # the coarse operator stalls or diverges (updates no longer at least
            # halve): switch to the fallback coarse operator and rebuild the
            # coarse values of the open slices so corrections and predictions
            # use one G
            if (
                self._fallback is not None and fallback_at is None and tol is not None and len(history) >= 2
                and (not np.all(np.isfinite(history[-1]))
                     or np.any(np.max(history[-1], axis=1) > 0.5 * np.max(history[-2], axis=1)))
            ):
                fallback_at = i + 1
                gname = "fallback"
                if not np.all(np.isfinite(history[-1])):
                    # non-finite coarse values reached some border points:
                    # those continue from their value before this
                    # iteration's sweep; the finite ones (among them the
                    # slice this iteration made exact) are kept
                    new = ws.U[1:, ..., :ws.fplan.ny]
                    bad = ~torch.isfinite(new).reshape(new.shape[0], -1).all(dim=1)
                    ws.U[1:][bad] = ws.old[bad]
                g = ws.coarse("fallback")
                ws.run_unit(("rebuild", i, gname), lambda i=i, g=g: ws.rebuild(i, g))

        ws.fplan.check_status()
        final = ws.fplan.unpack(ws.U[S], B, esize=8)
        out = {
            "final": final,
            "trajectory": None,
            "t": np.array([t1]),
            "d_t": t1 - t0,
            "iterations": iterations,
            "norm_history": history,
            "border_points": ws.U,
        }
        if self._trajectory != "final":
            out.update(self._fine_trajectory(ws.fplan, ws.U, ws.U_start, ws.f_in, S, B, ws.n_f, t_interval,
                                             ws.t_offsets, ws.fes, ws.fcomp, ws))
        self.last_stats = {
            "iterations": iterations.tolist(),
            "norm_history": [h.tolist() for h in history],
            "fallback_at_iteration": fallback_at,
            "eager_units": list(ws.eager_units),
        }
        return out

    def _callable_check(self, fplan, U, old, b, S) -> bool:
        new = fplan.unpack(U[1:, b].contiguous(), S, esize=8).cpu().numpy()
        prev = fplan.unpack(old[:, b].contiguous(), S, esize=8).cpu().numpy()
        return bool(self._termination_condition(prev, new))

    def _fine_trajectory(self, fplan, U, U_start, f_in, S, B, n_f, t_interval, t_offsets, fes, fcomp, ws=None):
        """The last iteration's fine sub-trajectories, each shifted so that it
        ends on the corrected border point (parareal_operator.py:190-193)."""
        import torch

        lib = _native.lib()
        stream = torch.cuda.current_stream().cuda_stream
        every = 1 if self._trajectory == "full" else int(self._trajectory)
        if n_f % every:
            raise ValueError(f"trajectory stride {every} must divide the fine steps per slice ({n_f})")
        n_save = n_f // every
        n_u = S * B * fplan.C * fplan.plane  # float64 elements of all border slices
        _native.check(lib.prml_pr_cast(U_start.data_ptr(), f_in.data_ptr(), fes, n_u, fcomp, stream), "cast")
        traj = fplan.new_state(n_save)  # (n_save, S*B, C, nx, pitch)
        if ws is not None and ws.fine_implicit:
            work = fplan.new_state(2) if every > 1 else None
            for j in range(S):
                fplan.run(ws.pf(f_in, j), traj.data_ptr() + j * B * fplan.inst * fes, n_f, float(ws.borders[j]),
                          self._f.d_t, save_every=every,
                          work=(ws.pf(work[0], j), ws.pf(work[1], j)) if work is not None else None,
                          traj_step_stride=S * B * fplan.inst, batch=B)
        else:
            fplan.run(f_in, traj, n_f, ws.t_base if ws is not None else 0.0, self._f.d_t, save_every=every,
                      t_offset_ptr=t_offsets.data_ptr(), bc_inst_slot_ptr=ws.bc_slot_ptr(0) if ws is not None else None)
        delta = torch.empty((S * B, fplan.C) + tuple(traj.shape[3:]), dtype=torch.float64, device=traj.device)
        _native.check(
            lib.prml_pr_end_delta(U[1:].data_ptr(), traj[n_save - 1].data_ptr(), fes, delta.data_ptr(), n_u, fcomp, stream),
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


class _Workspace:
    """Device buffers of one batched Parareal problem, kept across solves of
    the same shape, plus the CUDA graphs of its work units (the initial
    coarse pass and every iteration), recorded on first use and replayed
    afterwards so that the sequential coarse sweep costs no host time per
    launch."""

    def __init__(self, op: "PararealOperator", cp, B: int, t0: float, t1: float, key):
        import torch

        self.op, self.cp, self.B, self.key = op, cp, B, key
        S = op._n_slices
        self.S = S
        delta_t = (t1 - t0) / S
        self.delta_t = delta_t
        self.n_f = int(round(delta_t / op._f.d_t))
        self.borders = np.linspace(t0, t1, S + 1)
        # time-dependent boundary conditions: one set of half-step tables over
        # [t0, t1] for the fine plan (and each coarse plan), every slice
        # reading it from its own start (per-instance table offsets); runs
        # then start at t0 with per-slice time offsets from t0
        self.dynamic = bool(cp.differential_equation.x_dimension) and not cp.are_all_boundary_conditions_static
        self.t_base = t0 if self.dynamic else 0.0
        # an implicit fine operator steps each slice by its own secant solves
        # (one run per open slice, at its start time); host-driven iterations
        # cannot be recorded, so the work units then run eagerly
        from ... import codegen

        self.fine_implicit = getattr(op._f, "integrator_kind", None) in codegen.IMPLICIT
        self.eager = self.fine_implicit or any(
            getattr(o, "integrator_kind", None) in codegen.IMPLICIT for o in (op._g, op._fallback) if o is not None)
        C = cp.differential_equation.y_dimension
        self.C = C
        fplan = op._f.plan(cp, S * B)
        self.fplan = fplan
        dev = fplan.device
        self.dev = dev
        self.inst = C * fplan.plane
        self.u_shape = (B, C, fplan.nx, fplan.pitch)
        self.fes = fplan.esize
        self.fcomp = self.inst if fplan.comp else 0
        self.f_slice = B * fplan.inst
        self.u_slice = B * self.inst
        f64 = torch.float64
        self.U = torch.empty((S + 1,) + self.u_shape, dtype=f64, device=dev)
        self.U_start = torch.empty_like(self.U)
        self.g_old = torch.empty((S,) + self.u_shape, dtype=f64, device=dev)
        self.corr = torch.zeros((S,) + self.u_shape, dtype=f64, device=dev)
        self.old = torch.empty((S,) + self.u_shape, dtype=f64, device=dev)
        self.f_in = fplan.new_state(1)[0]
        self.f_end = fplan.new_state(1)[0]
        self.f_work = fplan.new_state(2) if self.n_f > 1 else None
        self.t_offsets = torch.tensor(np.repeat(self.borders[:-1] - self.t_base, B), dtype=f64, device=dev)
        self.bc_slots = None
        if self.dynamic:
            fplan.preset_tables(t0, op._f.d_t, S * self.n_f)
            self.bc_slots = torch.tensor(np.repeat(2 * self.n_f * np.arange(S), B).astype(np.int32), device=dev)
        self.active = torch.ones(B, dtype=torch.int32, device=dev)
        self.chunks = max(1, min(64, (fplan.nx * fplan.ny) // 4096))
        self.partial = torch.empty(_native.lib().prml_pr_norm_scratch_elems(S, B, C, self.chunks), dtype=f64, device=dev)
        self.norms = torch.empty((B, C), dtype=f64, device=dev)
        self._coarse = {}
        self.graphs = {}
        self.eager_units = []

    # ---- helpers
    def pu(self, t, j=0):
        return t.data_ptr() + j * self.u_slice * 8

    def pf(self, t, j=0):
        return t.data_ptr() + j * self.f_slice * self.fes

    @staticmethod
    def stream():
        import torch

        return torch.cuda.current_stream().cuda_stream

    def coarse(self, which: str) -> "_CoarseSlot":
        slot = self._coarse.get(which)
        if slot is None:
            g = self.op._g if which == "g" else self.op._fallback
            n_g = int(round(self.delta_t / g.d_t))
            prop = self.op._make_coarse(g, self.cp, self.B, n_g)
            if self.dynamic:
                plan = getattr(prop, "plan", None)
                if plan is None:
                    raise NotImplementedError("time-dependent boundary conditions need an FDM coarse operator")
                plan.preset_tables(float(self.borders[0]), g.d_t, self.S * n_g)
            slot = _CoarseSlot(self, prop)
            self._coarse[which] = slot
        return slot

    def bc_slot_ptr(self, first_slice: int) -> Optional[int]:
        """Device address of the fine launch's per-instance table offsets
        from slice ``first_slice`` on (None for static boundary conditions)."""
        if self.bc_slots is None:
            return None
        return self.bc_slots.data_ptr() + first_slice * self.B * 4

    def pack_y0(self, y0) -> None:
        """Initial states: a float64 host array or a CUDA float64 tensor
        (e.g. from ``gaussian_initial_states``), (batch, *vertices, C)."""
        import torch

        if isinstance(y0, torch.Tensor):
            y = y0.to(device=self.dev, dtype=torch.float64).contiguous()
        else:
            y = torch.from_numpy(np.ascontiguousarray(y0, dtype=np.float64)).to(self.dev)
        self.fplan.pack_device(y, self.U[0], esize=8)

    def reset(self) -> None:
        self.corr.zero_()
        self.active.fill_(1)

    def run_unit(self, key, fn) -> None:
        """Runs fn's launches, from a recorded CUDA graph when graphs are on."""
        import torch

        if not self.op._use_graphs or self.eager:
            fn()
            return
        graph = self.graphs.get(key)
        if graph is None:
            # first use runs eagerly: kernels get loaded and tuned, lazily
            # allocated workspaces exist, nothing host-synchronising is recorded
            fn()
            self.graphs[key] = "warm"
            return
        if graph == "eager":
            fn()
            return
        if graph == "warm":
            try:
                graph = self._record(fn)
            except Exception:  # a unit that cannot be recorded keeps running eagerly
                torch.cuda.synchronize()
                self.graphs[key] = "eager"
                self.eager_units.append(key)
                fn()
                return
            self.graphs[key] = graph
        graph.replay()

    def _record(self, fn):
        import torch

        graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(graph, stream=side):
                fn()
        torch.cuda.current_stream().wait_stream(side)
        return graph

    # ---- work units
    def init_sweep(self, g: "_CoarseSlot") -> None:
        """U_{j+1} = G(U_j) over all slices (corrections are zero)."""
        g.cast_in(0)
        for j in range(self.S):
            g.step(j, 0)

    def iteration(self, i: int, g: "_CoarseSlot", with_norm: bool) -> None:
        lib, chk, st = _native.lib(), _native.check, self.stream()
        S, B, inst, u_slice = self.S, self.B, self.inst, self.u_slice
        act = self.active.data_ptr()
        pu, pf = self.pu, self.pf
        # border points at the start of this iteration, per live instance
        chk(lib.prml_pr_copy(pu(self.U, 0), pu(self.U_start, 0), (S + 1) * u_slice, inst, act, B, st), "copy")
        # fine sweep over the slices that can still change (j >= i), batched
        m = S - i
        chk(lib.prml_pr_cast(pu(self.U, i), pf(self.f_in, i), self.fes, m * u_slice, self.fcomp, st), "cast")
        w = self.f_work
        if self.fine_implicit:
            for j in range(i, S):
                self.fplan.run(pf(self.f_in, j), pf(self.f_end, j), self.n_f, float(self.borders[j]),
                               self.op._f.d_t, save_every=self.n_f,
                               work=(pf(w[0], j), pf(w[1], j)) if w is not None else None, batch=B)
        else:
            self.fplan.run(
                pf(self.f_in, i), pf(self.f_end, i), self.n_f, self.t_base, self.op._f.d_t, save_every=self.n_f,
                work=(pf(w[0], i), pf(w[1], i)) if w is not None else None,
                batch=m * B, t_offset_ptr=self.t_offsets.data_ptr() + i * B * 8, bc_inst_slot_ptr=self.bc_slot_ptr(i),
            )
        chk(lib.prml_pr_correct(pf(self.f_end, i), self.fes, pu(self.g_old, i), pu(self.corr, i), m * u_slice,
                                inst, act, B, self.fcomp, st), "correct")
        chk(lib.prml_pr_copy(pu(self.U, 1), pu(self.old, 0), S * u_slice, inst, 0, B, st), "copy")
        # sequential coarse sweep
        chk(lib.prml_pr_advance(None, g.es, pu(self.g_old, i), pu(self.corr, i), pu(self.U, i + 1),
                                g.inp.data_ptr(), u_slice, inst, act, B, g.comp, st), "advance")
        for j in range(i + 1, S):
            g.step(j, act)
        if with_norm:
            fp = self.fplan
            chk(lib.prml_pr_update_norm(pu(self.U, 1), pu(self.old, 0), S, B, self.C, fp.nx, fp.ny, fp.pitch,
                                        self.chunks, self.partial.data_ptr(), self.norms.data_ptr(), st), "norm")

    def rebuild(self, i: int, g: "_CoarseSlot") -> None:
        """g_old[j] = G(U_j) for the open slices j > i (``old`` is scratch here)."""
        lib, chk, st = _native.lib(), _native.check, self.stream()
        act = self.active.data_ptr()
        for j in range(i + 1, self.S):
            g.cast_in(j)
            g.prop(g.inp, g.out, float(self.borders[j]))
            chk(lib.prml_pr_advance(g.out.data_ptr(), g.es, self.pu(self.g_old, j), self.pu(self.corr, j),
                                    self.pu(self.old, j), None, self.u_slice, self.inst, act, self.B, g.comp, st),
                "coarse rebuild")


class _CoarseSlot:
    """A coarse propagator with its own input/output states."""

    def __init__(self, ws: _Workspace, prop):
        import torch

        self.ws = ws
        self.prop = prop
        self.es = 8 if prop.dtype == "f64" else 4
        self.comp = ws.inst if prop.dtype == "f32c" else 0
        planes = 2 * ws.C if prop.dtype == "f32c" else ws.C
        shp = (ws.B, planes, ws.fplan.nx, ws.fplan.pitch)
        tdt = torch.float64 if prop.dtype == "f64" else torch.float32
        self.inp = torch.empty(shp, dtype=tdt, device=ws.dev)
        self.out = torch.empty(shp, dtype=tdt, device=ws.dev)

    def cast_in(self, j: int) -> None:
        ws = self.ws
        _native.check(_native.lib().prml_pr_cast(ws.pu(ws.U, j), self.inp.data_ptr(), self.es, ws.u_slice, self.comp,
                                                 ws.stream()), "cast")

    def step(self, j: int, act: int) -> None:
        """U_{j+1} = G(U_j) + corr_j, with G(U_j) kept in g_old[j]."""
        ws = self.ws
        self.prop(self.inp, self.out, float(ws.borders[j]))
        _native.check(
            _native.lib().prml_pr_advance(self.out.data_ptr(), self.es, ws.pu(ws.g_old, j), ws.pu(ws.corr, j),
                                          ws.pu(ws.U, j + 1), self.inp.data_ptr(), ws.u_slice, ws.inst,
                                          act, ws.B, self.comp, ws.stream()),
            "advance",
        )
