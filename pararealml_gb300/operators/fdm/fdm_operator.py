"""GPU drop-in for the reference's ``FDMOperator``.

Same constructor and contract as ``pararealml/operators/fdm/fdm_operator.py:
26-77``: ``FDMOperator(integrator, differentiator, d_t).solve(ivp)`` returns a
``Solution`` holding y at every time step after t0, vertex-oriented.  The
step loop, the stage arithmetic, the stencils and the constraint fills run as
one fused sm_103a kernel per step (``csrc/fdm_step.cuh``), generated from the
equation's ``symbolic_equation_system`` and compiled at run time.

GB300-side keyword-only options:

* ``dtype``: ``float64`` (default; matches the reference to ~1e-12 relative)
  or ``float32`` (the bandwidth-optimal path; its error against the float64
  result is reported by the tests and the benchmark).
* ``trajectory``: ``"full"`` (default, every step like the reference),
  ``"final"`` (only the last state) or an int k (every k-th step).  Anything
  but ``"full"`` returns fewer time points than the reference does.
* ``keep_on_device``: return the trajectory as a CUDA tensor inside the
  ``Solution`` (``solution.device_y``) and copy to the host only on demand.
* implicit integrators (``BackwardEulerMethod``, ``CrankNicolsonMethod``)
  run in float64 only: each step is the reference's element-wise secant
  solve (``numerical_integrator.py:135-270``) over right-hand-side kernel
  evaluations, with scipy.optimize.newton's warnings and error.
* ``op_order``: ``"fused"`` (default) or ``"reference"``.  Fused order
  evaluates the Cartesian Laplacian as one neighbour sum, uses explicit
  multiply-adds and combines the integrator's stages from unscaled slopes
  (a stage-invariant RK4 step is y + dt f): about half the floating-point
  operations of the reference's numpy order, each result within a few
  roundings of it.  ``"reference"`` keeps numpy's operation order and
  rounding (products with reciprocals aside).
* ``multi_round``: also build the multi-round kernels of the equation
  (every step of several batched solves in one cooperative launch with a
  grid barrier between steps; ``engine.MultiRun``), used by the ensemble
  solver.
* ``jacobi_max_iterations``: cap on the iterations of each step's
  anti-Laplacian solve (LHS.Y_LAPLACIAN components; the reference has none
  and loops until the change is at most the differentiator's ``tol``);
  reaching it raises ``ConvergenceError``.

LHS.Y_LAPLACIAN components are solved after every step by a device Jacobi
loop (``csrc/prml_jacobi.cu``) from an initial estimate drawn, like the
reference's (``numerical_differentiator.py:910-911``), from numpy's global
generator: under the same ``np.random.seed`` both draw the same estimates.
"""

from __future__ import annotations

from typing import Optional, Union

import numpy as np

from ...engine import StencilPlan, normalize_dtype, to_host
from ...codegen import lower_problem
from ...operator import Operator, discretize_time_domain
from ...solution import Solution
from .numerical_differentiator import check_differentiator
from .numerical_integrator import implicit_settings, integrator_kind


class FDMOperator(Operator):
    def __init__(
        self,
        integrator,
        differentiator,
        d_t: float,
        *,
        dtype=None,
        trajectory: Union[str, int] = "full",
        keep_on_device: bool = False,
        tile=None,
        max_ctas: int = 0,
        jacobi_max_iterations: int = 1_000_000,
        op_order: str = "fused",
        multi_round: bool = False,
    ):
        super().__init__(d_t, True)
        self._multi_round = bool(multi_round)
        if op_order not in ("fused", "reference"):
            raise ValueError("op_order must be 'fused' or 'reference'")
        self._op_order = op_order
        if jacobi_max_iterations < 1:
            raise ValueError("jacobi_max_iterations must be positive")
        self._jacobi_max_iterations = int(jacobi_max_iterations)
        self._max_ctas = max_ctas
        self._integrator = integrator
        self._differentiator = differentiator
        self._kind = integrator_kind(integrator)
        check_differentiator(differentiator)
        self._dtype = normalize_dtype(dtype)
        if not (trajectory in ("full", "final") or (isinstance(trajectory, int) and trajectory >= 1)):
            raise ValueError("trajectory must be 'full', 'final' or a positive int stride")
        self._trajectory = trajectory
        self._keep_on_device = keep_on_device
        self._tile = tile
        self._plans = {}

    @property
    def dtype(self) -> str:
        return self._dtype

    @property
    def integrator_kind(self) -> int:
        return self._kind

    def plan(self, cp, batch: int = 1) -> StencilPlan:
        """The (cached) stencil plan of this operator for ``cp`` and ``batch``."""
        key = (id(cp), batch)
        entry = self._plans.get(key)
        if entry is None or entry[0] is not cp:
            plan = StencilPlan(lower_problem(cp), self._kind, self._dtype, batch, self._tile,
                               op_order=self._op_order, multi=self._multi_round)
            plan.limit_ctas(self._max_ctas)
            plan.jacobi_tol = float(self._differentiator._tol)
            plan.jacobi_max_iterations = self._jacobi_max_iterations
            if plan.implicit is not None:
                plan.implicit = implicit_settings(self._integrator)
            entry = (cp, plan)
            if len(self._plans) > 8:
                self._plans.clear()
            self._plans[key] = entry
        return entry[1]

    def save_every(self, n_steps: int) -> int:
        if self._trajectory == "full":
            return 1
        if self._trajectory == "final":
            return max(n_steps, 1)
        k = int(self._trajectory)
        if n_steps % k:
            raise ValueError(f"trajectory stride {k} must divide the number of steps ({n_steps})")
        return k

    def solve(self, ivp, parallel_enabled: bool = True) -> Solution:
        cp = ivp.constrained_problem
        t = discretize_time_domain(ivp.t_interval, self._d_t)
        n_steps = len(t) - 1
        if n_steps == 0:
            raise ValueError("length of t coordinates must be greater than 0")
        y0 = _initial_state(cp, float(t[0]), ivp.initial_condition.discrete_y_0(True))
        plan = self.plan(cp, 1)
        state0 = plan.new_state(1)
        plan.pack(y0[np.newaxis], state0[0])
        every = self.save_every(n_steps)
        n_save = n_steps // every
        traj = plan.new_state(n_save)
        plan.run(state0[0], traj, n_steps, float(t[0]), self._d_t, every)
        y = plan.unpack(traj, n_save)
        plan.check_status()
        t_out = t[every::every]
        if self._keep_on_device:
            return Solution(ivp, t_out, y, vertex_oriented=True, d_t=self._d_t * every)
        # a fresh array only this solution refers to: no second copy
        return Solution(ivp, t_out, to_host(y), vertex_oriented=True, d_t=self._d_t * every, copy=False)

    def solve_into(self, ivp, out, chunk_saves: Optional[int] = None) -> Solution:
        """``solve`` with the trajectory written into the caller's float64
        host tensor ``out`` of shape (n_saved, *vertices, C), preferably in
        pinned memory: saved steps are streamed to it in chunks while the
        next chunk computes (``StencilPlan.run_to_host``), so neither the
        device nor the host needs a second full-size copy.  The returned
        Solution's ``discrete_y()`` is a view of ``out``."""
        import torch

        cp = ivp.constrained_problem
        t = discretize_time_domain(ivp.t_interval, self._d_t)
        n_steps = len(t) - 1
        if n_steps == 0:
            raise ValueError("length of t coordinates must be greater than 0")
        y0 = _initial_state(cp, float(t[0]), ivp.initial_condition.discrete_y_0(True))
        plan = self.plan(cp, 1)
        state0 = plan.new_state(1)
        plan.pack(y0[np.newaxis], state0[0])
        every = self.save_every(n_steps)
        n_save = n_steps // every
        shape = (n_save,) + tuple(y0.shape)
        if tuple(out.shape) != shape:
            raise ValueError(f"out must have shape {shape}, got {tuple(out.shape)}")
        plan.run_to_host(state0[0], out.view((n_save, 1) + tuple(y0.shape)), n_steps, float(t[0]), self._d_t,
                         every, chunk_saves)
        plan.check_status()
        return Solution(ivp, t[every::every], out.numpy(), vertex_oriented=True, d_t=self._d_t * every, copy=False)

    def solve_device(self, cp, y0_device, t0: float, n_steps: int, save_every: Optional[int] = None):
        """Device-level solve: float64 (batch, *vertices, C) input, device states out.

        Returns the trajectory as device states of shape (n_saved, batch, C, nx, pitch).
        """
        batch = y0_device.shape[0]
        plan = self.plan(cp, batch)
        state0 = plan.new_state(1)
        if not cp.are_all_boundary_conditions_static and cp.differential_equation.x_dimension:
            import torch

            y0_device = torch.from_numpy(
                np.stack([_initial_state(cp, t0, y) for y in y0_device.cpu().numpy()])
            ).to(y0_device.device)
        plan.pack_device(y0_device, state0[0])
        every = save_every or self.save_every(n_steps)
        traj = plan.new_state(n_steps // every)
        plan.run(state0[0], traj, n_steps, t0, self._d_t, every)
        return traj


def _initial_state(cp, t0: float, y0) -> np.ndarray:
    """The initial state as the reference steps from it: with time-dependent
    boundary conditions the y constraints at t0 are applied first
    (``fdm_operator.py:56-63``); with static ones the state is used as is
    (not copied: every caller only reads it)."""
    from ...constraint import apply_constraints_along_last_axis

    if not cp.differential_equation.x_dimension or cp.are_all_boundary_conditions_static:
        return np.asarray(y0, dtype=np.float64)
    y = np.array(y0, dtype=np.float64, copy=True)
    constraints = cp.create_y_vertex_constraints(cp.create_boundary_constraints(True, t0)[0])
    return apply_constraints_along_last_axis(constraints, y)
