"""``Solution.y`` / ``discrete_y`` / ``diff`` against the reference's own
outputs (golden fixture ``solution_interp_diff`` made by
``tests/golden/make_golden.py`` with the unmodified reference,
pararealml/solution.py:114-258).

CPU: this package's ``Solution`` built on the reference's stored
trajectories reproduces the reference's interpolations and differences
exactly.  GPU: the same calls on this package's own solves match within
1e-12 relative L2 (the trajectories themselves match to rounding).
"""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import load, rel_l2

FIX = "solution_interp_diff"


def _ivp():
    return problems.diffusion_2d(ns, n=16, t_end=0.2)


def _check(fe, rk, gold, exact):
    def same(a, b):
        if exact:
            assert np.array_equal(a, b)
        else:
            assert a.shape == b.shape and rel_l2(a, b) < 1e-12

    x = gold["x"]
    same(fe.y(x), gold["y_linear"])
    same(fe.y(x, "nearest"), gold["y_nearest"])
    same(fe.discrete_y(False), gold["cells"])
    d = fe.diff([rk])
    assert np.allclose(d.matching_time_points, gold["diff_t"], rtol=0, atol=1e-15)
    assert len(d.differences) == 1
    same(d.differences[0], gold["diff_0"])


def test_solution_on_reference_trajectories_matches_reference():
    gold = load(FIX)
    ivp = _ivp()
    fe = ns.Solution(ivp, gold["t_fe"], gold["y_fe"], vertex_oriented=True, d_t=0.01)
    rk = ns.Solution(ivp, gold["t_rk"], gold["y_rk"], vertex_oriented=True, d_t=0.02)
    _check(fe, rk, gold, exact=True)
    with pytest.raises(ValueError):
        fe.diff([])


@pytest.mark.gpu
def test_solution_of_gpu_solves_matches_reference():
    from pararealml_gb300.operators import fdm

    gold = load(FIX)
    ivp = _ivp()
    fe = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.01).solve(ivp)
    rk = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.02).solve(ivp)
    assert rel_l2(fe.discrete_y(), gold["y_fe"]) < 1e-12 and rel_l2(rk.discrete_y(), gold["y_rk"]) < 1e-12
    _check(fe, rk, gold, exact=False)
