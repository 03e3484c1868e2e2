"""Failure paths on the GPU, exercised without faulting it (needs a GB300).

Every wait inside the kernels is bounded (%globaltimer) and reports through
a device status word that the host turns into an exception; the context
stays usable.  The tests make a wait run out the allowed way: a staging
barrier armed for a copy that is never issued (the step kernels'
``wait_probe`` 1) and a grid barrier that waits for one arrival more than
the grid has (the multi-round kernel's ``wait_probe`` 2), each with a 1 ms
bound.  The Parareal fallback is forced from the host: a coarse propagator
whose output is overwritten with NaN.
"""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import rel_l2
from pararealml_gb300.operators import fdm
from pararealml_gb300.operators.parareal import PararealOperator

pytestmark = pytest.mark.gpu


def _rk4(d_t, **kw):
    return fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), d_t, **kw)


def test_step_kernel_wait_runs_out_reports_and_recovers():
    ivp = problems.cahn_hilliard_2d(ns, n=40, length=10.0, t_end=0.004)
    cp = ivp.constrained_problem
    want = _rk4(0.001, trajectory="final").solve(ivp).discrete_y()[-1]
    op = _rk4(0.001, trajectory="final", tile=(16, 32, 128))
    plan = op.plan(cp, 1)
    s0 = plan.new_state(1)
    plan.pack(ivp.initial_condition.discrete_y_0(True)[np.newaxis], s0[0])
    end = plan.new_state(1)
    plan.params.wait_limit_ns = 1_000_000  # 1 ms
    plan.params.wait_probe = 1
    try:
        plan.run(s0[0], end, 4, 0.0, 0.001, 4)
        with pytest.raises(RuntimeError, match="timed out"):
            plan.check_status()
    finally:
        plan.params.wait_probe = 0
        plan.params.wait_limit_ns = 0
    # the status was cleared and the plan (and the context) stay usable
    plan.run(s0[0], end, 4, 0.0, 0.001, 4)
    plan.check_status()
    got = plan.unpack(end[0], 1).cpu().numpy()[0]
    assert rel_l2(got, want) < 1e-12


def test_multi_round_grid_barrier_runs_out_reports_and_recovers():
    from pararealml_gb300.ensemble import EnsembleSolver

    ivps = [problems.cahn_hilliard_2d(ns, n=24, length=6.0, t_end=0.006, seed=s) for s in (1, 2)]
    solver = EnsembleSolver(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), dtype="float64", use_graph=False,
                            launch="persistent")
    solver.setup(ivps, [0.001, 0.001])
    assert solver.tile is not None
    plan0 = solver._multi.plan0
    solver.advance()
    good = solver.final_states()
    for g in solver._multi.groups:
        g["plan"].params.wait_limit_ns = 1_000_000
        g["plan"].params.wait_probe = 2
    solver._multi._desc.clear()  # re-encode the descriptors with the probe
    try:
        solver.advance()
        with pytest.raises(RuntimeError, match="timed out"):
            plan0.check_status()
    finally:
        for g in solver._multi.groups:
            g["plan"].params.wait_limit_ns = 0
            g["plan"].params.wait_probe = 0
        solver._multi._desc.clear()
    solver.advance()
    again = solver.final_states()
    for a, b in zip(good, again):
        assert np.array_equal(a, b)


class _NaNAfter:
    """A coarse operator (FDM forward Euler) whose propagator output is
    overwritten with NaN from its ``after``-th call on: a coarse step that
    blew up, injected on the host."""

    def __init__(self, d_t, after):
        self._fe = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), d_t)
        self.d_t = d_t
        self.vertex_oriented = True
        self.after = after
        self.calls = 0

    def coarse_propagator(self, cp, batch, n_steps):
        from pararealml_gb300.operators.parareal.parareal_operator import FDMCoarsePropagator

        inner = FDMCoarsePropagator(self._fe, cp, batch, n_steps)
        outer = self

        class _Prop:
            dtype = inner.dtype

            def __call__(self, src, dst, t_start):
                inner(src, dst, t_start)
                outer.calls += 1
                if outer.calls >= outer.after:
                    dst.fill_(float("nan"))

        return _Prop()


def test_parareal_falls_back_when_the_coarse_step_returns_nan():
    """The NaN coarse values make the update norms non-finite after the
    second iteration: the operator puts back the border points that turned
    non-finite (keeping the slice that iteration made exact), switches to
    the fallback coarse operator, and after S iterations equals the fine
    solution as Parareal must."""
    ivp = problems.cahn_hilliard_2d(ns, n=16, length=4.0, t_end=0.04)
    S = 4
    f = _rk4(0.001)
    fine_only = f.solve(ivp).discrete_y()[-1]
    # initial sweep: S coarse calls; iteration 0 sweep: S - 1; NaN from the
    # first call of iteration 1's sweep on
    g = _NaNAfter(0.002, after=2 * S)
    fallback = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.002)
    op = PararealOperator(f, g, 1e-13, S, n_slices=S, trajectory="final", fallback=fallback, use_graphs=False)
    got = op.solve(ivp).discrete_y()[-1]
    assert op.last_stats["fallback_at_iteration"] == 2
    assert not np.all(np.isfinite(op.last_stats["norm_history"][1]))
    assert np.isfinite(got).all()
    assert rel_l2(got, fine_only) < 1e-12
