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


def test_mixed_size_ensemble_equals_individual_solves():
    ivps, d_ts = problems.shallow_water_ensemble(ns, n_instances=9, sizes=(16, 32, 48), t_end=0.5, seed=11)
    solver = EnsembleSolver(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), dtype="float64")
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
