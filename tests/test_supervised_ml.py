"""SupervisedMLOperator host logic against the reference's own outputs (CPU).

``tests/golden/sml_cases.npz`` holds the reference's ``generate_data``
results (its RK4 FDMOperator as the oracle, ``problems.sml_perturbation``
drawing from numpy's global generator seeded per job), a least-squares model
fitted by its ``fit_model`` and that model's ``solve`` trajectory
(pararealml/operators/ml/supervised/supervised_ml_operator.py).  Here the
oracle is the numpy restatement of the reference's FDM solver, so the data
must match to rounding (1e-12), and everything downstream of the data
(split, fit, scores, auto-regressive solve) exactly.  The GPU oracle is
checked in ``test_gpu_supervised_ml.py``.
"""

import os
import sys

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from oracle import fdm as orc
from pararealml_gb300.operator import Operator, discretize_time_domain
from pararealml_gb300.operators.ml import SupervisedMLOperator, mean_squared_error, train_test_indices
from pararealml_gb300.solution import Solution

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from make_golden import SML_CASES, SML_D_T, SML_ORACLE_D_T  # noqa: E402

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "sml_cases.npz"))


class NumpyFDMOracle(Operator):
    """The oracle restatement of the reference's RK4 FDMOperator as an
    Operator (test infrastructure: the checker, not the product)."""

    def __init__(self, d_t):
        super().__init__(d_t, True)

    def solve(self, ivp, parallel_enabled=True):
        cp = ivp.constrained_problem
        y = orc.fdm_solve(cp, ivp.initial_condition.discrete_y_0(True), ivp.t_interval, self.d_t, "rk4")
        t = discretize_time_domain(ivp.t_interval, self.d_t)[1:]
        return Solution(ivp, t, y, vertex_oriented=True, d_t=self.d_t)


@pytest.mark.parametrize("name", sorted(SML_CASES))
def test_generate_data_matches_the_reference(name):
    builder, kw, op_kw, gen_kw = SML_CASES[name]
    ivp = getattr(problems, builder)(ns, **kw)
    op = SupervisedMLOperator(SML_D_T, **op_kw)
    x, y = op.generate_data(ivp, NumpyFDMOracle(SML_ORACLE_D_T), perturbation_function=problems.sml_perturbation,
                            **gen_kw)
    want_x, want_y = GOLD[f"{name}_x"], GOLD[f"{name}_y"]
    assert x.shape == want_x.shape and y.shape == want_y.shape
    assert np.allclose(x, want_x, rtol=1e-12, atol=1e-14)
    assert np.allclose(y, want_y, rtol=1e-12, atol=1e-14)


def test_fit_model_and_solve_match_the_reference():
    """Same split (numpy's global generator under seed 3), same least-squares
    fit, same scores, and the same auto-regressive trajectory."""
    x, y = GOLD["ar_x"], GOLD["ar_y"]
    op = SupervisedMLOperator(SML_D_T, True)
    np.random.seed(3)
    train, test = op.fit_model(problems.AffineModel(), (x, y), test_size=0.25)
    assert np.array_equal(op.model.coef_, GOLD["fit_coef"])
    assert [train, test] == list(GOLD["fit_scores"])
    sol = op.solve(problems.sml_diffusion_1d(ns))
    assert np.array_equal(sol.discrete_y(), GOLD["solve_y"])
    assert np.allclose(sol.t_coordinates, [0.05, 0.1, 0.15])


def test_split_and_score_equal_scikit_learn():
    sk = pytest.importorskip("sklearn.model_selection")
    metrics = pytest.importorskip("sklearn.metrics")
    rng = np.random.default_rng(0)
    x = rng.random((37, 3))
    y = rng.random((37, 2))
    for test_size in (0.2, 0.25, 0.5):
        np.random.seed(11)
        want = sk.train_test_split(x, y, test_size=test_size)
        np.random.seed(11)
        tr, te = train_test_indices(len(x), test_size)
        for a, b in zip(want, (x[tr], x[te], y[tr], y[te])):
            assert np.array_equal(a, b)
    p = rng.random((37, 2))
    assert mean_squared_error(y, p) == metrics.mean_squared_error(y, p)


def test_argument_checks_like_the_reference():
    with pytest.raises(ValueError, match="time variant"):
        SupervisedMLOperator(0.1, True, auto_regressive=False)
    with pytest.raises(ValueError, match="time invariant"):
        SupervisedMLOperator(0.1, True, time_variant=True, input_d_t=True)
    op = SupervisedMLOperator(0.05, True)
    ivp = problems.sml_diffusion_1d(ns)
    with pytest.raises(ValueError, match="no model"):
        op.solve(ivp)
    oracle = NumpyFDMOracle(0.01)
    with pytest.raises(ValueError, match="iterations"):
        op.generate_data(ivp, oracle, 0, problems.sml_perturbation)
    with pytest.raises(ValueError, match="jobs"):
        op.generate_data(ivp, oracle, 1, problems.sml_perturbation, n_jobs=0)
    with pytest.raises(ValueError, match="seeds"):
        op.generate_data(ivp, oracle, 2, problems.sml_perturbation, n_jobs=2, seeds=[1])
    with pytest.raises(ValueError, match="perturbed y shape"):
        op.generate_data(ivp, oracle, 1, lambda t, y: y[:-1])


def test_repeat_on_error_draws_again():
    """A solve that fails once is retried with a fresh perturbation (and a
    warning) when repeat_on_error is set; without it the error propagates."""

    class Flaky(NumpyFDMOracle):
        calls = 0

        def solve(self, ivp, parallel_enabled=True):
            Flaky.calls += 1
            if Flaky.calls == 2:
                raise RuntimeError("injected oracle failure")
            return super().solve(ivp, parallel_enabled)

    ivp = problems.sml_diffusion_1d(ns)
    op = SupervisedMLOperator(SML_D_T, True)
    with pytest.warns(UserWarning, match="injected oracle failure"):
        x, y = op.generate_data(ivp, Flaky(SML_ORACLE_D_T), 1, problems.sml_perturbation, repeat_on_error=True)
    assert Flaky.calls == 4 and x.shape[0] == 3 * 13
    Flaky.calls = 0
    with pytest.raises(RuntimeError, match="injected"):
        op.generate_data(ivp, Flaky(SML_ORACLE_D_T), 1, problems.sml_perturbation)


def test_fields_layout_holds_the_same_pairs():
    """layout='fields': the same (input state, target state) pairs as the
    reference's rows, one pair per sub-IVP."""
    ivp = problems.diffusion_2d(ns, n=6, t_end=0.15)
    op = SupervisedMLOperator(SML_D_T, True)
    oracle = NumpyFDMOracle(SML_ORACLE_D_T)
    np.random.seed(0)
    xr, yr = op.generate_data(ivp, oracle, 2, problems.sml_perturbation)
    np.random.seed(0)
    xf, yf = op.generate_data(ivp, oracle, 2, problems.sml_perturbation, layout="fields")
    n_pts = 7 * 7
    assert xf.shape == (6, 7, 7, 1) and yf.shape == (6, 7, 7, 1)
    for k in range(6):
        assert np.array_equal(xr[k * n_pts, :n_pts], xf[k].reshape(-1))
        assert np.array_equal(yr[k * n_pts:(k + 1) * n_pts, 0], yf[k].reshape(-1))
