"""The CPU oracle against the reference's golden outputs and known answers.

The oracle (``oracle/fdm.py``) is the checker for the GPU path, so it is
pinned first: against fixtures produced by running the reference itself
(``tests/golden``) and against the known-answer tests of the reference's own
suite (``tests/operators/fdm/test_numerical_differentiator.py`` and
``test_numerical_integrator.py``), restated here.
"""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import FDM_CASES, ORACLE_INTEGRATOR, PARAREAL_CASES, load, oracle_integrator, rel_l2
from oracle import fdm as orc


class _C:
    """Minimal constraint (values + mask) for the stencil known answers."""

    def __init__(self, values, mask):
        self.values = np.asarray(values, dtype=float)
        self.mask = np.asarray(mask, dtype=bool)


@pytest.mark.parametrize("name", sorted(FDM_CASES))
def test_oracle_matches_reference_fdm(name):
    builder, kw, integ, d_t = FDM_CASES[name]
    gold = load(name)
    ivp = builder(ns, **kw)
    y0 = ivp.initial_condition.discrete_y_0(True)
    assert np.array_equal(y0, gold["y0"]) or rel_l2(y0, gold["y0"]) < 1e-15
    np.random.seed(problems.JACOBI_SEED)  # initial estimates of the Jacobi solves
    kind, kw = oracle_integrator(integ)
    traj = orc.fdm_solve(ivp.constrained_problem, y0, ivp.t_interval, d_t, kind, **kw)
    assert traj.shape[0] == int(gold["n_steps"])
    got = traj[gold["steps"] - 1]
    assert rel_l2(got, gold["y"]) < 1e-13


@pytest.mark.parametrize("name", sorted(PARAREAL_CASES))
def test_oracle_matches_reference_parareal(name):
    builder, kw, fi, fdt, gi, gdt, ranks, tol, max_it = PARAREAL_CASES[name]
    gold = load(name)
    ivp = builder(ns, **kw)
    cp = ivp.constrained_problem
    y0 = ivp.initial_condition.discrete_y_0(True)

    def runner(integ, d_t, keep):
        def run(y, ta, tb):
            n = int(round((tb - ta) / d_t))
            return orc.fdm_solve(cp, y, (ta, ta + n * d_t), d_t, ORACLE_INTEGRATOR[integ], keep=keep)

        return run

    _, iters, traj = orc.parareal_solve(
        cp, y0, ivp.t_interval, ranks, runner(fi, fdt, "final"), runner(gi, gdt, "final"),
        tol, max_it, fine_traj=runner(fi, fdt, "full"),
    )
    assert traj.shape[0] == int(gold["n_steps"])
    assert rel_l2(traj[gold["steps"] - 1], gold["y"]) < 1e-12
    assert 1 <= iters <= min(ranks, max_it)


# ---- known answers restated from the reference's differentiator tests
Y3x3x2 = np.array(
    [
        [[2.0, 4.0], [4.0, 8.0], [-3.0, 2.0]],
        [[6.0, 4.0], [4.0, 4.0], [5.0, -1.0]],
        [[2.0, 6.0], [8.0, 2.0], [-7.0, 7.0]],
    ]
)


def test_kat_gradient():
    exp = np.array(
        [
            [[1.5, 1.0], [1.0, 1.0], [1.25, -0.25]],
            [[0.0, 0.5], [1.0, -1.5], [-1.0, 1.25]],
            [[-1.5, -1.0], [-1.0, -1.0], [-1.25, 0.25]],
        ]
    )
    assert np.allclose(orc.gradient(Y3x3x2, (2.0, 1.0), 0), exp)


def test_kat_1d_constrained_gradient():
    y = np.array([[2.0, 4.0], [4.0, 8.0], [-3.0, 2.0], [-3.0, 2.0]])
    dbc = np.empty((1, 2), dtype=object)
    dbc[0, 0] = (None, _C([-9999.0], [True]))
    dbc[0, 1] = (_C([9999.0], [True]), None)
    exp = np.array([[1.0, 9999.0], [-1.25, -0.5], [-1.75, -1.5], [-9999.0, -0.5]])
    assert np.allclose(orc.gradient(y, (2.0,), 0, dbc), exp)


def test_kat_2d_constrained_gradient():
    dbc = np.empty((2, 2), dtype=object)
    dbc[0, 0] = (None, _C(np.full(2, -9999.0), [[True], [False], [True]]))
    dbc[0, 1] = (_C(np.full(1, 9999.0), [[False], [True], [False]]), None)
    exp = np.array(
        [
            [[1.5, 1.0], [1.0, 9999.0], [1.25, -0.25]],
            [[0.0, 0.5], [1.0, -1.5], [-1.0, 1.25]],
            [[-9999.0, -1.0], [-1.0, -1.0], [-9999.0, 0.25]],
        ]
    )
    assert np.allclose(orc.gradient(Y3x3x2, (2.0, 1.0), 0, dbc), exp)


def test_kat_hessian():
    y = np.array([[[4.0], [8.0], [2.0]], [[4.0], [4.0], [-1.0]], [[6.0], [2.0], [7.0]]])
    exp = np.array([[[-1.0], [-3.0], [-1.25]], [[0.5], [0.5], [2.75]], [[-2.0], [0.0], [-3.75]]])
    assert np.allclose(orc.hessian(y, (2.0, 1.0), 0, 0), exp)


def test_kat_1d_constrained_hessian():
    y = np.array([[2.0], [4.0], [-3.0], [-3.0]])
    dbc = np.empty((1, 1), dtype=object)
    dbc[0, 0] = (_C([0.0], [True]), _C([], [False]))
    exp = np.array([[1.0], [-2.25], [1.75], [0.75]])
    assert np.allclose(orc.hessian(y, (2.0,), 0, 0, dbc), exp)


def test_kat_2d_constrained_hessian():
    dbc = np.empty((2, 2), dtype=object)
    dbc[0, 1] = (_C(np.full(2, -2.0), [[True], [True], [False]]), _C(np.full(1, 0.0), [[False], [False], [True]]))
    exp = np.array(
        [
            [[0.5, 2.0], [-1.0, 0.0], [2.75, -1.25]],
            [[-2.0, 0.5], [1.0, 0.5], [-5.0, 2.75]],
            [[0.5, -2.0], [-3.0, 0.0], [4.75, -4.0]],
        ]
    )
    assert np.allclose(orc.hessian(Y3x3x2, (2.0, 2.0), 0, 0, dbc), exp)


def test_kat_mixed_hessian():
    y = np.array([[[2.0], [4.0], [-3.0]], [[6.0], [4.0], [5.0]], [[2.0], [8.0], [-7.0]]])
    exp = np.array([[[2.0], [-0.5], [-2.0]], [[2.0], [-2.0], [-2.0]], [[-2.0], [0.5], [2.0]]])
    assert np.allclose(orc.hessian(y, (1.0, 0.5), 0, 1), exp)


def test_kat_divergence():
    exp = np.array([[[5.0], [1.5], [0.5]], [[1.0], [0.75], [-3.0]], [[-2.5], [-1.75], [-3.0]]])
    assert np.allclose(orc.divergence(Y3x3x2, (1.0, 2.0)), exp)


def test_kat_laplacian():
    y = np.array(
        [
            [[2.0, 4.0], [4.0, 8.0], [2.0, 4.0]],
            [[6.0, 4.0], [4.0, 4.0], [10.0, -4.0]],
            [[2.0, 6.0], [8.0, 2.0], [-2.0, 4.0]],
        ]
    )
    exp = np.array(
        [
            [[0.5, -1.0], [-5.0, -11.0], [1.5, -3.0]],
            [[-10.0, -3.5], [9.0, -7.5], [-21.0, 16.0]],
            [[4.5, -12.0], [-19.0, 6.0], [15.5, -9.0]],
        ]
    )
    assert np.allclose(orc.laplacian(y, (2.0, 1.0)), exp)


def test_stencil_needs_three_points():
    with pytest.raises(ValueError):
        orc.derivative(np.zeros((2, 3, 1)), 1.0, 0, [None])


# ---------------------------------------------------------------- anti-Laplacian
# The reference's anti-Laplacian tests (tests/operators/fdm/
# test_numerical_differentiator.py:527-667, 937-1025, 1600-1660) take a random
# field y with Dirichlet faces, its Laplacian, and require the Jacobi solve at
# tol 1e-12 to give back y.  The same cases, restated on the oracle (plus a
# spherical one, which the reference does not test).


def _field_constraint(shape, faces):
    """Full-field constraint from an ordered list of ((axis, side), value):
    later entries win at edges and corners, like the reference's arrays."""
    value = np.full(tuple(shape) + (1,), np.nan)
    for (axis, side), v in faces:
        sl = [slice(None)] * (len(shape) + 1)
        sl[axis] = 0 if side == 0 else -1
        value[tuple(sl)] = v
    mask = ~np.isnan(value)
    return _C(value[mask], mask)


def _face_neumann(shape, axis, value):
    """Upper-face derivative constraint of one component along ``axis``."""
    fshape = list(shape) + [1]
    fshape[axis] = 1
    mask = np.ones(fshape, dtype=bool)
    return _C(np.full(int(mask.sum()), value), mask)


_ALL_FACES = {2: [((0, 0), 1.0), ((0, 1), 2.0), ((1, 0), 3.0), ((1, 1), 42.0)]}
_ALL_FACES[3] = _ALL_FACES[2] + [((2, 0), 41.0), ((2, 1), 40.0)]

ANTI_LAPLACIAN_KATS = {
    # name: (coordinate system, bounds, steps, derivative constraints)
    "cartesian_2d": ("CARTESIAN", [(0.0, 0.95), (0.0, 0.475)], [0.05, 0.025], False),
    "cartesian_1d_neumann": ("CARTESIAN", [(0.0, 0.95)], [0.05], True),
    "cartesian_2d_neumann": ("CARTESIAN", [(0.0, 0.95), (0.0, 0.475)], [0.05, 0.025], True),
    "polar": ("POLAR", [(1.0, 2.9), (0.0, 0.95)], [0.1, 0.05], False),
    "polar_neumann": ("POLAR", [(1.0, 2.9), (0.0, 0.95)], [0.1, 0.05], True),
    "cylindrical": ("CYLINDRICAL", [(1.0, 1.7), (0.0, 0.35), (0.0, 1.4)], [0.1, 0.05, 0.2], False),
    "spherical": ("SPHERICAL", [(1.0, 1.7), (0.0, 0.35), (0.3, 1.0)], [0.1, 0.05, 0.1], False),
}


def anti_laplacian_kat(name, seed=7):
    """(y, Laplacian, y constraints, derivative constraints, d_x, grids, cs)
    of one known-answer case; the Laplacian uses the same derivative
    constraints as the solve."""
    cs, bounds, steps, neumann = ANTI_LAPLACIAN_KATS[name]
    mesh = ns.Mesh(bounds, steps, getattr(ns.CoordinateSystem, cs))
    shape = tuple(mesh.vertices_shape)
    d = len(shape)
    rng = np.random.default_rng(seed)
    y = rng.random(shape + (2,))
    if neumann:
        # component 0: Dirichlet on the lower faces only; component 1 on all
        # faces; Neumann -3 on the upper face of axis 0 (and 0 on the upper
        # face of axis 1) of component 0, like the reference's cases
        c0 = _field_constraint(shape, [((a, 0), [1.0, 3.0][a]) for a in range(d)])
        c1 = _field_constraint(shape, [((0, 0), -2.0), ((0, 1), 2.0)] + ([((1, 0), 5.0), ((1, 1), 4.0)] if d > 1 else []))
        dbc = np.empty((d, 2), dtype=object)
        dbc.fill(None)
        for a in range(d):
            dbc[a, 0] = (None, _face_neumann(shape, a, [-3.0, 0.0][a]))
        yc = [c0, c1]
    else:
        c = _field_constraint(shape, _ALL_FACES[d])
        dbc = None
        yc = [c, c]
    for i, c in enumerate(yc):
        orc.apply_mask(c.values, c.mask, y[..., i: i + 1])
    grids = mesh.vertex_coordinate_grids
    d_x = tuple(mesh.d_x)
    lap = orc.laplacian(y, d_x, dbc) if cs == "CARTESIAN" else orc.laplacian_cs(cs, y, d_x, dbc, grids)
    return y, lap, yc, dbc, d_x, grids, cs


@pytest.mark.parametrize("name", sorted(ANTI_LAPLACIAN_KATS))
def test_kat_anti_laplacian(name):
    y, lap, yc, dbc, d_x, grids, cs = anti_laplacian_kat(name)
    np.random.seed(3)
    anti = orc.anti_laplacian(cs, lap, d_x, yc, dbc, grids, 1e-12)
    back = orc.laplacian(anti, d_x, dbc) if cs == "CARTESIAN" else orc.laplacian_cs(cs, anti, d_x, dbc, grids)
    assert np.allclose(back, lap)
    assert np.allclose(anti, y)


def test_anti_laplacian_stops_at_the_first_change_within_tol():
    """``while diff > tol`` from diff = inf: a tolerance above the first
    change stops after one iteration, tol = inf runs none (the result is the
    constrained initial estimate)."""
    y, lap, yc, dbc, d_x, grids, cs = anti_laplacian_kat("cartesian_2d")
    for tol, n in ((1e9, 1), (np.inf, 0)):
        counter = []
        out = orc.anti_laplacian(cs, lap, d_x, yc, dbc, grids, tol, y_init=np.zeros_like(y), counter=counter)
        assert counter == [n]
    assert np.array_equal(out, orc.apply_y_constraints(yc, np.zeros_like(y)))


# ---------------------------------------------------------------- secant
def test_secant_restatement_matches_scipy_newton():
    """The implicit integrators' solver (ImplicitMethod._solve,
    numerical_integrator.py:157-176) is scipy.optimize.newton without a
    derivative on the whole array; the oracle's restatement gives the same
    roots, iteration-dependent results, warnings and error on polynomial,
    flat (zero-derivative), coupled and capped problems."""
    import warnings

    scipy_opt = pytest.importorskip("scipy.optimize")
    rng = np.random.default_rng(0)
    for trial in range(120):
        n = int(rng.integers(2, 30))
        a, b, c = rng.normal(size=n), rng.normal(size=n), rng.normal(size=n)
        m = rng.normal(size=(n, n)) * 0.1
        kind = trial % 4
        funcs = [
            lambda x: a * x ** 3 + b * x - c,
            lambda x: np.tanh(x) - 0.3 * c,
            lambda x: np.where(np.abs(x) > 5, 0.0, x - c),
            lambda x: x + m @ np.sin(x) - c,
        ]
        f = funcs[kind]
        x0 = rng.normal(size=n) * 2
        maxit = int(rng.integers(3, 60))
        try:
            with warnings.catch_warnings(record=True) as w:
                warnings.simplefilter("always")
                want = scipy_opt.newton(f, x0, tol=1.48e-8, maxiter=maxit)
            want_w, want_err = [str(x.message) for x in w], None
        except RuntimeError as e:
            want, want_w, want_err = None, [], str(e)
        try:
            got, _, got_w = orc.secant_solve(f, x0, 1.48e-8, maxit)
            got_err = None
        except RuntimeError as e:
            got, got_w, got_err = None, None, str(e)
        assert want_err == got_err
        if want_err is None:
            assert np.array_equal(want, got, equal_nan=True)
            assert (got_w is None) == (not want_w) and (got_w is None or got_w in want_w)


# The reference's implicit-integrator known answers
# (tests/operators/fdm/test_numerical_integrator.py:141-268), restated:
# dy/dt = 5 y + t^2 from y(1) = 1 with dt = 0.5 has the backward Euler step
# (y0 + dt (t0 + dt)^2) / (1 - 5 dt); Crank-Nicolson with a = 0 is forward
# Euler and with a = 1 backward Euler.


def _ode_f(t, y):
    return 5.0 * y + t ** 2


def _end_constraint(shape, value=999.0):
    v = np.full(shape[:-1] + (1,), np.nan)
    v[0] = v[-1] = value
    mask = ~np.isnan(v)
    return _C(v[mask], mask)


@pytest.mark.parametrize("constrained", [False, True])
def test_kat_backward_euler(constrained):
    y0 = np.ones((5, 1)) if constrained else np.array([1.0])
    con = [_end_constraint(y0.shape)] if constrained else None
    want = (y0 + 0.5 * 1.5 ** 2) / (1.0 - 5 * 0.5)
    if constrained:
        orc.apply_y_constraints(con, want)
    got, _, warning = orc.implicit_integral(y0, 1.0, 0.5, _ode_f, lambda t: con)
    assert np.allclose(got, want) and warning is None


@pytest.mark.parametrize("constrained", [False, True])
def test_kat_crank_nicolson(constrained):
    y0 = np.ones((5, 1)) if constrained else np.array([1.0])
    con = [_end_constraint(y0.shape)] if constrained else None
    t0, dt, a = 1.0, 0.5, 0.5
    # y1 = y0 + a dt (5 y1 + t1^2) + (1 - a) dt (5 y0 + t0^2)
    want = (y0 + a * dt * (t0 + dt) ** 2 + (1 - a) * dt * (5 * y0 + t0 ** 2)) / (1.0 - a * 5 * dt)
    if constrained:
        orc.apply_y_constraints(con, want)
    got, _, warning = orc.implicit_integral(y0, t0, dt, _ode_f, lambda t: con, a, True)
    assert np.allclose(got, want) and warning is None


def test_kat_crank_nicolson_limits():
    y0 = np.array([1.0])
    fe = y0 + 0.1 * _ode_f(1.0, y0)
    cn0, _, _ = orc.implicit_integral(y0, 1.0, 0.1, _ode_f, lambda t: None, 0.0, True)
    assert np.allclose(cn0, fe)
    be, _, _ = orc.implicit_integral(y0, 1.0, 0.1, _ode_f, lambda t: None)
    cn1, _, _ = orc.implicit_integral(y0, 1.0, 0.1, _ode_f, lambda t: None, 1.0, True)
    assert np.allclose(cn1, be)
