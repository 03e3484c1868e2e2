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
    """parareal_operator.py:114-123; also a coarse step of 1e-2 for
    0.125-long slices (32 slices of [0, 4]) is rejected exactly as the
    reference does."""
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


def test_preset_boundary_table_slots():
    """Runs on a preset time-dependent table grid (Parareal slices) start at
    the half-step table of their start time; runs off the grid, with another
    step size or past its end build their own tables (None)."""
    import types

    from pararealml_gb300.engine import StencilPlan

    plan = types.SimpleNamespace(_preset=(0.3, 0.001, 40))
    slot = lambda t0, dt, n: StencilPlan._preset_slot(plan, t0, dt, n)  # noqa: E731
    borders = np.linspace(0.3, 0.34, 5)
    assert [slot(t, 0.001, 10) for t in borders[:-1]] == [0, 20, 40, 60]
    assert slot(0.3, 0.002, 10) is None  # another step size
    assert slot(0.3005, 0.001, 10) is None  # on a half step, not a step
    assert slot(0.33, 0.001, 11) is None  # past the end of the grid
    assert slot(0.29, 0.001, 1) is None  # before its start
    plan._preset = None
    assert slot(0.3, 0.001, 10) is None
