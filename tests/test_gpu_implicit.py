"""GPU parity of the implicit integrators (backward Euler, Crank-Nicolson).

The reference solves each step with scipy.optimize.newton (the vectorised
secant method) on the whole state (numerical_integrator.py:135-270).  Bars:
float64 results within REL_F64 = 1e-12 relative L2 of the reference's own
outputs (golden fixtures, test_gpu_fdm.py) and of the oracle; the same
secant iteration count per step; the same warnings and error as
scipy.optimize.newton when the iteration cap or the tolerance is reached.
"""

import warnings

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


def _oracle(ivp, kind, d_t, **kw):
    cp = ivp.constrained_problem
    st = orc.FDMStepper(cp, kind, d_t, **kw)
    t = orc.time_grid(ivp.t_interval, d_t)
    y = np.array(ivp.initial_condition.discrete_y_0(True))
    if st.dynamic:
        y = orc.apply_y_constraints(st.yc(t[0]), y)
    out = []
    for i in range(len(t) - 1):
        y = st.step(t[i], y)
        out.append(y)
    return np.stack(out), st


@pytest.mark.parametrize("case", [
    ("diffusion_2d", dict(n=24, t_end=0.08), "BackwardEulerMethod", (), "be", {}, 0.01),
    ("cahn_hilliard_2d", dict(n=20, length=5.0, t_end=0.006), "CrankNicolsonMethod", (0.3,), "cn", {"cn_a": 0.3}, 0.001),
    ("convection_diffusion_1d", dict(n=40, t_end=0.1), "CrankNicolsonMethod", (), "cn", {}, 0.01),
    ("diffusion_3d_mixed", dict(n=(7, 9, 11), t_end=0.006), "BackwardEulerMethod", (), "be", {}, 0.002),
])
def test_trajectory_and_secant_iterations_match_the_oracle(case):
    builder, kw, integ, args, kind, okw, d_t = case
    ivp = getattr(problems, builder)(ns, **kw)
    op = fdm.FDMOperator(getattr(fdm, integ)(*args), fdm.ThreePointCentralDifferenceMethod(), d_t)
    got = op.solve(ivp).discrete_y()
    want, st = _oracle(ivp, kind, d_t, **okw)
    assert rel_l2(got, want) < REL_F64
    plan = op.plan(ivp.constrained_problem, 1)
    assert [i[0] for i in plan.secant_iterations] == st.secant_iterations


def test_batched_instances_stop_like_separate_solves():
    """Instances with different initial states in one plan: each stops at
    its own secant iteration, so each equals its own oracle solve."""
    import torch

    base = problems.diffusion_2d(ns, n=24, t_end=0.05)
    cp = base.constrained_problem
    rng = np.random.default_rng(3)
    y0 = np.stack([base.initial_condition.discrete_y_0(True) * s + 0.05 * rng.random((25, 25, 1))
                   for s in (1.0, 0.3, 2.0)])
    op = fdm.FDMOperator(fdm.BackwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.01)
    traj = op.solve_device(cp, torch.tensor(y0, device="cuda"), 0.0, 5)
    plan = op.plan(cp, 3)
    got = plan.unpack(traj, 5 * 3).cpu().numpy().reshape(5, 3, 25, 25, 1)
    its = np.array(plan.secant_iterations)
    for b in range(3):
        st = orc.FDMStepper(cp, "be", 0.01)
        y = y0[b].copy()
        want = []
        for k in range(5):
            y = st.step(k * 0.01, y)
            want.append(y)
        assert rel_l2(got[:, b], np.stack(want)) < REL_F64
        assert list(its[:, b]) == st.secant_iterations
    assert len({tuple(its[:, b]) for b in range(3)}) > 1


@pytest.mark.parametrize("tol,max_iterations", [(0.0, 2), (1e-15, 3), (1e-3, 1)])
def test_warnings_and_error_like_scipy_newton(tol, max_iterations):
    """Iteration cap and tolerance outcomes: the device raises RuntimeError
    exactly when the oracle's restatement of scipy.optimize.newton does, and
    otherwise warns with the same message (or not at all)."""
    ivp = problems.diffusion_2d(ns, n=16, t_end=0.01)
    cp = ivp.constrained_problem
    y0 = ivp.initial_condition.discrete_y_0(True)

    def oracle_outcome():
        st = orc.FDMStepper(cp, "be", 0.01, secant_tol=tol, secant_maxiter=max_iterations)
        with warnings.catch_warnings(record=True) as w:
            warnings.simplefilter("always")
            try:
                y = st.step(0.0, np.array(y0))
            except RuntimeError as e:
                return "error", str(e), None
        return "ok", [str(x.message) for x in w], y

    want = oracle_outcome()
    op = fdm.FDMOperator(fdm.BackwardEulerMethod(tol, max_iterations), fdm.ThreePointCentralDifferenceMethod(), 0.01)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        try:
            y = op.solve(ivp).discrete_y()[0]
            got = ("ok", [str(x.message) for x in w if issubclass(x.category, RuntimeWarning)], y)
        except RuntimeError as e:
            got = ("error", str(e), None)
    assert got[0] == want[0]
    if want[0] == "error":
        assert got[1] == want[1]
    else:
        assert got[0] == "ok"
        # the oracle's warnings come from its own secant (no stacklevel
        # filtering): compare the messages
        assert sorted(set(got[1])) == sorted(set(m for m in want[1]))
        assert rel_l2(got[2], want[2]) < REL_F64


def test_float32_is_refused_and_an_implicit_coarse_step_serves_parareal():
    """Implicit steps run in float64 only; as Parareal's coarse operator a
    backward Euler step works, and with as many iterations as slices the
    result is the fine solution."""
    ivp = problems.diffusion_2d(ns, n=16, t_end=0.02)
    with pytest.raises(NotImplementedError):
        fdm.FDMOperator(fdm.BackwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.01,
                        dtype="float32").solve(ivp)
    from pararealml_gb300.operators.parareal import PararealOperator

    f = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.001)
    g = fdm.FDMOperator(fdm.BackwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.01)
    got = PararealOperator(f, g, 1e-14, 2, n_slices=2, trajectory="final").solve(ivp).discrete_y()[-1]
    want = f.solve(ivp).discrete_y()[-1]
    assert rel_l2(got, want) < 1e-12


def test_reference_crank_nicolson_conserves_density():
    """tests/operators/fdm/test_fdm_operator.py:63-93 on the device: 1D
    diffusion (D = 5) on [0, 500] with steps 0.1, zero-flux faces, a Gaussian
    bump, Crank-Nicolson dt 1e-3 to t = 20 (20000 secant-solved steps): the
    total density of every step equals the initial one."""
    diff_eq = ns.DiffusionEquation(1, 5.0)
    mesh = ns.Mesh([(0.0, 500.0)], [0.1])
    bc = ns.NeumannBoundaryCondition(lambda x, t: np.zeros((len(x), 1)), is_static=True)
    cp = ns.ConstrainedProblem(diff_eq, mesh, [(bc, bc)])
    ic = ns.GaussianInitialCondition(cp, [(np.array([250]), np.array([[250.0]]))], [1000.0])
    ivp = ns.InitialValueProblem(cp, (0.0, 20.0), ic)
    y_0_sum = np.sum(ic.discrete_y_0(True))
    solution = fdm.FDMOperator(fdm.CrankNicolsonMethod(), fdm.ThreePointCentralDifferenceMethod(), 1e-3).solve(ivp)
    y = solution.discrete_y()
    assert y.shape == (20000, 5001, 1)
    assert np.allclose(np.sum(y, axis=tuple(range(1, y.ndim))), y_0_sum)
