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


def test_large_copies_split_over_threads_equal_numpy_copies():
    """discrete_y's copy of a large trajectory (split over host threads) is
    an independent array equal to np.copy's, for sizes that do and do not
    divide evenly among the threads."""
    from pararealml_gb300 import solution as sol_mod

    rng = np.random.default_rng(3)
    for n in (sol_mod._PARALLEL_COPY_BYTES // 8 + 13, 3 * sol_mod._PARALLEL_COPY_BYTES // 8 + 1):
        a = rng.standard_normal(n).reshape(-1, 1) if n % 2 else rng.standard_normal(n)
        b = sol_mod._copy(a)
        assert b.shape == a.shape and np.array_equal(b, a) and not np.shares_memory(a, b)
        b[0] += 1.0
        assert b[0] != a[0]
    small = rng.standard_normal(10)
    assert np.array_equal(sol_mod._copy(small), small)
