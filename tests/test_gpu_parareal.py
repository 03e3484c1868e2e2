"""GPU parity of batched single-GPU Parareal (needs a GB300).

Bars: float64 fine/coarse solvers reproduce the reference's own multi-rank
Parareal output (golden fixtures made by running the reference's
PararealOperator on 4 thread-ranks) to REL_F64 = 1e-12 relative L2; batched
instances reproduce per-instance serial replays of the reference algorithm
(``oracle.fdm.parareal_solve``) to the same bar with the same iteration
counts.
"""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import ORACLE_INTEGRATOR, PARAREAL_CASES, load, rel_l2
from oracle import fdm as orc
from pararealml_gb300.operators import fdm
from pararealml_gb300.operators.parareal import PararealOperator

pytestmark = pytest.mark.gpu

REL_F64 = 1e-12


def _fdm(integ, d_t, **kw):
    return fdm.FDMOperator(getattr(fdm, integ)(), fdm.ThreePointCentralDifferenceMethod(), d_t, **kw)


@pytest.mark.parametrize("name", sorted(PARAREAL_CASES))
def test_matches_reference_multi_rank_parareal(name):
    builder, kw, fi, fdt, gi, gdt, ranks, tol, max_it = PARAREAL_CASES[name]
    gold = load(name)
    ivp = builder(ns, **kw)
    op = PararealOperator(_fdm(fi, fdt), _fdm(gi, gdt), tol, max_it, n_slices=ranks)
    y = op.solve(ivp).discrete_y()
    assert y.shape[0] == int(gold["n_steps"])
    assert rel_l2(y[gold["steps"] - 1], gold["y"]) < REL_F64


def _oracle_parareal(cp, y0, t_interval, S, fi, fdt, gi, gdt, tol, max_it):
    def runner(integ, d_t):
        def run(y, ta, tb):
            n = int(round((tb - ta) / d_t))
            return orc.fdm_solve(cp, y, (ta, ta + n * d_t), d_t, ORACLE_INTEGRATOR[integ], keep="final")

        return run

    u, iters, _ = orc.parareal_solve(cp, y0, t_interval, S, runner(fi, fdt), runner(gi, gdt), tol, max_it)
    return u, iters


def test_batched_gaussians_match_per_instance_replays():
    rng = np.random.default_rng(3)
    base = problems.diffusion_2d(ns, n=24, t_end=0.8)
    cp = base.constrained_problem
    ivps = []
    for _ in range(5):
        mean = rng.uniform(3.0, 7.0, 2)
        s = rng.uniform(0.4, 1.0)
        ic = ns.GaussianInitialCondition(cp, [(mean, s * np.eye(2))], [2 * np.pi * s])
        ivps.append(ns.InitialValueProblem(cp, (0.0, 0.8), ic))
    S, fi, fdt, gi, gdt, tol = 8, "RK4", 0.01, "ForwardEulerMethod", 0.025, 1e-7
    op = PararealOperator(_fdm(fi, fdt), _fdm(gi, gdt), tol, n_slices=S, trajectory="final")
    sols = op.solve_batch(ivps)
    for b, ivp in enumerate(ivps):
        y0 = ivp.initial_condition.discrete_y_0(True)
        u, iters = _oracle_parareal(cp, y0, (0.0, 0.8), S, fi, fdt, gi, gdt, tol, 100)
        assert op.last_stats["iterations"][b] == iters
        assert rel_l2(sols[b].discrete_y()[-1], u[-1]) < REL_F64


def test_float32_fine_and_coarse_with_fp64_correction():
    builder, kw, fi, fdt, gi, gdt, ranks, tol, max_it = PARAREAL_CASES["parareal_diffusion"]
    gold = load("parareal_diffusion")
    ivp = builder(ns, **kw)
    op = PararealOperator(_fdm(fi, fdt, dtype="float32"), _fdm(gi, gdt, dtype="float32"), tol, max_it, n_slices=ranks)
    y = op.solve(ivp).discrete_y()
    assert rel_l2(y[gold["steps"] - 1], gold["y"]) < 1e-5


def test_strided_trajectory_and_serial_mode():
    builder, kw, fi, fdt, gi, gdt, ranks, tol, max_it = PARAREAL_CASES["parareal_diffusion"]
    ivp = builder(ns, **kw)
    full = PararealOperator(_fdm(fi, fdt), _fdm(gi, gdt), tol, max_it, n_slices=ranks).solve(ivp).discrete_y()
    strided = PararealOperator(_fdm(fi, fdt), _fdm(gi, gdt), tol, max_it, n_slices=ranks, trajectory=10).solve(ivp)
    assert np.allclose(strided.discrete_y(), full[9::10], rtol=0, atol=1e-14)
    serial = PararealOperator(_fdm(fi, fdt), _fdm(gi, gdt), tol, n_slices=ranks).solve(ivp, parallel_enabled=False)
    assert np.array_equal(serial.discrete_y(), _fdm(fi, fdt).solve(ivp).discrete_y())


def test_callable_and_per_component_termination():
    ivp = problems.cahn_hilliard_2d(ns, n=16, length=4.0, t_end=0.04)
    f, g = _fdm("RK4", 0.001), _fdm("ForwardEulerMethod", 0.002)
    calls = []

    def never(old, new):
        calls.append((old.shape, new.shape))
        return False

    op = PararealOperator(f, g, never, 3, n_slices=4, trajectory="final")
    op.solve(ivp)
    assert len(calls) == 3 and calls[0][0] == (4, 17, 17, 2)
    op = PararealOperator(f, g, [1e-9, 1e-9], n_slices=4, trajectory="final")
    op.solve(ivp)
    assert op.last_stats["iterations"] == [4] or op.last_stats["iterations"][0] <= 4


def test_graph_replayed_solves_equal_the_eager_solve():
    """The first solve runs eagerly, the second records CUDA graphs of every
    work unit, later solves replay them: all must give the same answer."""
    builder, kw, fi, fdt, gi, gdt, ranks, tol, max_it = PARAREAL_CASES["parareal_diffusion"]
    gold = load("parareal_diffusion")
    ivp = builder(ns, **kw)
    op = PararealOperator(_fdm(fi, fdt), _fdm(gi, gdt), tol, max_it, n_slices=ranks)
    ys = [op.solve(ivp).discrete_y() for _ in range(3)]
    assert np.array_equal(ys[0], ys[1]) and np.array_equal(ys[1], ys[2])
    assert rel_l2(ys[2][gold["steps"] - 1], gold["y"]) < REL_F64


def test_compensated_fine_and_coarse_reach_the_float64_answer():
    builder, kw, fi, fdt, gi, gdt, ranks, tol, max_it = PARAREAL_CASES["parareal_diffusion"]
    gold = load("parareal_diffusion")
    ivp = builder(ns, **kw)
    op = PararealOperator(_fdm(fi, fdt, dtype="float32c"), _fdm(gi, gdt, dtype="float32c"), tol, max_it, n_slices=ranks)
    y = op.solve(ivp).discrete_y()
    assert rel_l2(y[gold["steps"] - 1], gold["y"]) < 1e-7
