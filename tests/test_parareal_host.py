"""Host-side argument checks of the Parareal operator (no GPU needed)."""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from pararealml_gb300.operators import fdm
from pararealml_gb300.operators.parareal import PararealOperator


def _ops(fdt=0.005, gdt=0.0125):
    f = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), fdt)
    g = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), gdt)
    return f, g


def test_step_sizes_must_divide_the_slices():
    """parareal_operator.py:114-123; also the stated config-3 coarse step
    (1e-2 for 0.125-long slices) is rejected exactly as the reference does."""
    ivp = problems.diffusion_2d(ns, n=8, t_end=4.0)
    f, _ = _ops(1e-4)
    g = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 1e-2)
    op = PararealOperator(f, g, 1e-6, n_slices=32)
    with pytest.raises(ValueError, match="coarse"):
        op.run(ivp.constrained_problem, ivp.initial_condition.discrete_y_0(True)[None], ivp.t_interval)
    f_bad = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.3)
    with pytest.raises(ValueError, match="fine"):
        PararealOperator(f_bad, g, 1e-6, n_slices=32).run(
            ivp.constrained_problem, ivp.initial_condition.discrete_y_0(True)[None], ivp.t_interval
        )


def test_tolerance_length_must_match_components():
    f, g = _ops()
    op = PararealOperator(f, g, [1e-6, 1e-6], n_slices=2)
    with pytest.raises(ValueError):
        op._tolerances(1)
    assert np.array_equal(op._tolerances(2), [1e-6, 1e-6])


def test_bad_arguments():
    f, g = _ops()
    with pytest.raises(ValueError):
        PararealOperator(f, g, 1e-6, n_slices=0)
    with pytest.raises(ValueError):
        PararealOperator(f, g, 1e-6, trajectory="every")
    ivp = problems.diffusion_2d(ns, n=8, t_end=1.0)
    with pytest.raises(ValueError):
        PararealOperator(f, g, 1e-6, 0, n_slices=4).run(
            ivp.constrained_problem, ivp.initial_condition.discrete_y_0(True)[None], ivp.t_interval
        )


def test_time_dependent_boundary_conditions_are_rejected_by_parareal():
    """The batched Parareal runs slices with different start times in one
    launch; time-dependent boundary tables per slice are not built, so it
    refuses such problems before touching the GPU."""
    ivp = problems.dynamic_bc_diffusion_1d(ns)
    f = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.5)
    g = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 2.5)
    op = PararealOperator(f, g, 1e-6, n_slices=4)
    with pytest.raises(NotImplementedError):
        op.solve(ivp)
