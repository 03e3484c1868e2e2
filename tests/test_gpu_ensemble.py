"""Uneven-size ensembles in one graph-recorded run (needs a GB300)."""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import rel_l2
from oracle import fdm as orc
from pararealml_gb300.ensemble import EnsembleSolver
from pararealml_gb300.operators import fdm

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("launch", ["persistent", "streams"])
def test_mixed_size_ensemble_equals_individual_solves(launch):
    """Both launch modes: one cooperative multi-round kernel over every
    group and step, and one launch per step and group on group streams."""
    ivps, d_ts = problems.shallow_water_ensemble(ns, n_instances=9, sizes=(16, 32, 48), t_end=0.5, seed=11)
    solver = EnsembleSolver(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), dtype="float64", launch=launch)
    solver.setup(ivps, d_ts)
    solver.advance()   # eager
    solver.advance()   # records the graph
    solver.advance()   # replays it
    got = solver.final_states()
    for ivp, d_t, y in zip(ivps, d_ts, got):
        op = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), d_t, trajectory="final")
        want = op.solve(ivp).discrete_y()[-1]
        assert rel_l2(y, want) < 1e-14
    y0 = ivps[0].initial_condition.discrete_y_0(True)
    want = orc.fdm_solve(ivps[0].constrained_problem, y0, ivps[0].t_interval, d_ts[0], "rk4", keep="final")
    assert rel_l2(got[0], want) < 1e-12


@pytest.mark.parametrize("dtype", ["float32", "float32c"])
def test_persistent_ensemble_single_stage_and_compensated(dtype):
    """The multi-round kernel on single-stage steps (Cahn-Hilliard RK4 is
    stage-invariant) with two mesh sizes and step counts: equal to the
    one-launch-per-step solves of each instance."""
    ivps, d_ts = [], []
    for n, t_end in ((24, 0.012), (40, 0.012)):
        for seed in (1, 2):
            ivps.append(problems.cahn_hilliard_2d(ns, n=n, length=n / 4.0, t_end=t_end, seed=seed))
            d_ts.append(0.001 if n == 24 else 0.0005)
    solver = EnsembleSolver(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), dtype=dtype, launch="persistent")
    solver.setup(ivps, d_ts)
    assert solver.tile is not None
    solver.advance()
    solver.advance()
    solver.advance()
    got = solver.final_states()
    for ivp, d_t, y in zip(ivps, d_ts, got):
        op = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), d_t, trajectory="final", dtype=dtype)
        want = op.solve(ivp).discrete_y()[-1]
        assert rel_l2(y, want) < 1e-6


def test_auto_launch_picks_one_form_and_matches():
    """The default launch times both forms once at setup and keeps the
    faster; either way the result is the per-instance solve's."""
    ivps, d_ts = problems.shallow_water_ensemble(ns, n_instances=6, sizes=(16, 32), t_end=0.5, seed=5)
    solver = EnsembleSolver(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), dtype="float64")
    solver.setup(ivps, d_ts)
    assert set(solver.stats) >= {"persistent_ms", "streams_ms"}
    solver.advance()
    solver.advance()
    for ivp, d_t, y in zip(ivps, d_ts, solver.final_states()):
        op = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), d_t, trajectory="final")
        assert rel_l2(y, op.solve(ivp).discrete_y()[-1]) < 1e-14
