"""GPU parity of the Jacobi anti-Laplacian (LHS.Y_LAPLACIAN rows).

The reference solves these rows after every step by Jacobi iteration from a
random estimate drawn from numpy's global generator
(numerical_differentiator.py:872-927, 1097-1186; fdm_operator.py:141-161).
Bars: with the same initial estimates the device solve takes the same
number of iterations as the oracle and its result is within REL_F64 = 1e-12
relative L2 (float64); full solves under the same ``np.random.seed`` match
the reference's own outputs (golden fixtures, test_gpu_fdm.py) and here the
reference's Navier-Stokes test assertions.
"""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import rel_l2
from oracle import fdm as orc
from pararealml_gb300 import _native
from pararealml_gb300.operators import fdm

pytestmark = pytest.mark.gpu

REL_F64 = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _built():
    _native.build()
    yield


def _plan(ivp, batch=1, dtype="float64", tol=1e-3):
    op = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(tol), 0.01, dtype=dtype)
    return op.plan(ivp.constrained_problem, batch)


def _device_solve(plan, lap, inits):
    """Runs the plan's anti-Laplacian on (batch, *V, n_lap) right-hand sides
    with the given initial estimates; returns the solution and the
    per-instance iteration counts."""
    low = plan.low
    batch = lap.shape[0]
    full = np.zeros(lap.shape[:-1] + (low.n_comp,))
    full[..., list(low.lap_idx)] = lap
    state = plan.new_state(1)
    plan.pack(full, state[0])
    it = iter(inits)
    plan.jacobi_init = lambda shape: next(it)
    plan.anti_laplacian(state[0])
    out = plan.unpack(state, batch).cpu().numpy()
    return out[..., list(low.lap_idx)], plan.jacobi_iterations[-1]


def _oracle_solve(ivp, lap, init, tol):
    cp = ivp.constrained_problem
    st = orc.FDMStepper(cp, "rk4", 0.01)
    lap_idx = st.rhs.lap_idx
    yc = st.yc(0.0)
    dyc = st.dyc(0.0)
    counter = []
    out = orc.anti_laplacian(st.rhs.cs, lap, st.rhs.d_x, None if yc is None else yc[lap_idx],
                             None if dyc is None else dyc[:, lap_idx], st.rhs.grids, tol, y_init=init,
                             counter=counter)
    return out, counter[0]


def _smooth_rhs(ivp, rng, scale=1.0):
    cp = ivp.constrained_problem
    grids = cp.mesh.vertex_coordinate_grids
    base = sum(np.sin((k + 1.3) * g) for k, g in enumerate(grids))
    return scale * (base + 0.1 * rng.standard_normal(base.shape))[..., None]


@pytest.mark.parametrize("key", sorted(problems._JACOBI_MESHES))
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_solve_matches_oracle_iteration_for_iteration(key, dtype):
    """Random initial estimates at tol 1e-3 (the reference's default): same
    iteration count as the oracle and the same result (float64 within
    1e-12; float32 within 1e-5, its rounding of the estimates)."""
    ivp = problems.jacobi_system(ns, key[0], key[1])
    rng = np.random.default_rng(11)
    lap = _smooth_rhs(ivp, rng)
    init = rng.random(lap.shape)
    want, n = _oracle_solve(ivp, lap, init, 1e-3)
    got, its = _device_solve(_plan(ivp, dtype=dtype), lap[None], [init])
    assert its == [n] or dtype == "float32"
    assert rel_l2(got[0], want) < (REL_F64 if dtype == "float64" else 1e-5)


def test_batched_instances_stop_independently():
    """Three instances with different right-hand sides and estimates: each
    stops at its own iteration (per-instance norms and stop flags)."""
    ivp = problems.jacobi_system(ns, "CARTESIAN", 2)
    rng = np.random.default_rng(5)
    laps = [_smooth_rhs(ivp, rng, s) for s in (1.0, 0.2, 3.0)]
    inits = [rng.random(laps[0].shape) * s for s in (1.0, 0.01, 2.0)]
    got, its = _device_solve(_plan(ivp, batch=3), np.stack(laps), inits)
    for b in range(3):
        want, n = _oracle_solve(ivp, laps[b], inits[b], 1e-3)
        assert its[b] == n
        assert rel_l2(got[b], want) < REL_F64
    assert len(set(its)) > 1


@pytest.mark.parametrize("mesh,dtype", [
    (([(0.0, 2.0), (-1.0, 1.5)], [2.0 / 300, 2.5 / 211]), "float64"),
    (([(0.0, 2.0), (-1.0, 1.5)], [2.0 / 300, 2.5 / 211]), "float32"),
    (([(0.0, 1.0), (0.0, 1.2), (0.0, 1.4)], [1.0 / 40, 1.2 / 45, 1.4 / 50]), "float64"),
    # planes too large to stage with a halo: the unstaged kernel
    (([(0.0, 1.0), (0.0, 1.0), (0.0, 1.0)], [1.0 / 19, 1.0 / 129, 1.0 / 129]), "float64"),
])
def test_many_ctas_per_instance(mesh, dtype):
    """Meshes large enough for many CTAs per instance (grid barrier, partial
    norms summed by every CTA, halo bands recomputed by neighbouring CTAs),
    random estimates and a tolerance of 2% of the first change, so the run
    takes tens of iterations."""
    dims = len(mesh[0])
    ivp = problems.jacobi_system(ns, "CARTESIAN", dims, mesh=mesh)
    rng = np.random.default_rng(9)
    lap = _smooth_rhs(ivp, rng)
    init = rng.random(lap.shape)
    one, _ = _oracle_solve(ivp, lap, init, 1e9)  # one iteration
    c = orc.FDMStepper(ivp.constrained_problem, "rk4", 0.01).yc(0.0)
    first_change = float(np.linalg.norm(one - orc.apply_y_constraints(c[[1]], init.copy())))
    tol = 0.02 * first_change
    want, n = _oracle_solve(ivp, lap, init, tol)
    plan = _plan(ivp, tol=tol, dtype=dtype)
    got, its = _device_solve(plan, lap[None], [init])
    assert n > 10
    if dtype == "float64":
        assert its == [n] and rel_l2(got[0], want) < REL_F64
    else:
        assert abs(its[0] - n) <= 1 and rel_l2(got[0], want) < 1e-4


def test_tolerance_edge_cases_and_iteration_cap():
    """tol = inf runs no iteration (the constrained estimate comes back);
    a cap below the needed count raises ConvergenceError and the plan stays
    usable."""
    ivp = problems.jacobi_system(ns, "CARTESIAN", 2)
    rng = np.random.default_rng(2)
    lap = _smooth_rhs(ivp, rng)
    init = rng.random(lap.shape)
    want, n = _oracle_solve(ivp, lap, init, np.inf)
    plan = _plan(ivp, tol=np.inf)
    plan.jacobi_tol = np.inf
    got, its = _device_solve(plan, lap[None], [init])
    assert n == 0 and its == [0]
    assert np.array_equal(got[0], want)
    plan.jacobi_tol = 0.0
    plan.jacobi_max_iterations = 7
    with pytest.raises(_native.ConvergenceError):
        _device_solve(plan, lap[None], [init])
    assert plan.jacobi_iterations[-1] == [-1]
    plan.jacobi_tol, plan.jacobi_max_iterations = 1e-3, 1_000_000
    want, n = _oracle_solve(ivp, lap, init, 1e-3)
    got, its = _device_solve(plan, lap[None], [init])
    assert its == [n] and rel_l2(got[0], want) < REL_F64


def test_kat_anti_laplacian_recovers_the_field():
    """The reference's known-answer structure (test_numerical_differentiator.py:
    527-667) on the device, with this problem's Dirichlet, Neumann and free
    faces: at tol 1e-12 the solve gives back the field whose Laplacian (with
    the same Neumann ghosts) was the right-hand side."""
    mesh = ([(0.0, 0.95), (0.0, 0.475)], [0.05, 0.025])
    ivp = problems.jacobi_system(ns, "CARTESIAN", 2, mesh=mesh)
    cp = ivp.constrained_problem
    rng = np.random.default_rng(4)
    y = rng.random(tuple(cp.mesh.vertices_shape) + (1,))
    st = orc.FDMStepper(cp, "rk4", 0.01)
    c = st.yc(0.0)[[1]]
    orc.apply_y_constraints(c, y)
    dbc = st.dyc(0.0)[:, [1]]
    lap = orc.laplacian(y, tuple(cp.mesh.d_x), dbc)
    got, _ = _device_solve(_plan(ivp, tol=1e-12), lap[None], [rng.random(y.shape)])
    assert np.allclose(got[0], y)
    assert np.allclose(orc.laplacian(got[0], tuple(cp.mesh.d_x), dbc), lap)


def test_reference_navier_stokes_assertions():
    """tests/operators/fdm/test_fdm_operator.py:136-170 on the device, and
    the full trajectory against the oracle under the same seed."""
    ivp = problems.navier_stokes_2d(ns)
    np.random.seed(problems.JACOBI_SEED)
    sol = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.25).solve(ivp)
    assert sol.vertex_oriented
    assert sol.d_t == 0.25
    assert sol.discrete_y().shape == (40, 11, 11, 4)
    assert sol.discrete_y(False).shape == (40, 10, 10, 4)
    np.random.seed(problems.JACOBI_SEED)
    want = orc.fdm_solve(ivp.constrained_problem, ivp.initial_condition.discrete_y_0(True), ivp.t_interval,
                         0.25, "rk4")
    assert rel_l2(sol.discrete_y(), want) < REL_F64


def test_same_seed_same_solution_and_generator_state():
    """Two solves under one seed agree bit for bit, and the solve consumes
    numpy's global generator exactly like the reference (one estimate per
    step), so the next draw after it matches the oracle's."""
    ivp = problems.jacobi_system(ns, "POLAR", 2)
    op = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.005)
    np.random.seed(1)
    a = op.solve(ivp).discrete_y()
    after_gpu = np.random.random()
    np.random.seed(1)
    b = op.solve(ivp).discrete_y()
    assert np.array_equal(a, b)
    np.random.seed(1)
    orc.fdm_solve(ivp.constrained_problem, ivp.initial_condition.discrete_y_0(True), ivp.t_interval, 0.005, "rk4")
    assert after_gpu == np.random.random()


def test_parareal_rejects_laplacian_rows():
    from pararealml_gb300.operators.parareal import PararealOperator

    ivp = problems.navier_stokes_2d(ns)
    f = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.25)
    g = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.5)
    with pytest.raises(NotImplementedError):
        PararealOperator(f, g, 1e-3).solve(ivp)
