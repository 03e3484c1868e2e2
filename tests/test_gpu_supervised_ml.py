"""SupervisedMLOperator with the GPU FDMOperator as the oracle, and the CNN
regressor behind its model contract (needs a GB300).

Bars: data generated through the GPU oracle equal the reference's own
``generate_data`` outputs (``tests/golden/sml_cases.npz``) within 1e-12,
through the one-solve-per-sub-IVP path and through the batched device
solves, which draw the perturbations in the reference's order.
"""

import os
import sys

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import rel_l2
from pararealml_gb300.learned import CNNRegressor
from pararealml_gb300.operators import fdm
from pararealml_gb300.operators.ml import SupervisedMLOperator
from pararealml_gb300.operators.parareal import PararealOperator

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from make_golden import SML_CASES, SML_D_T, SML_ORACLE_D_T  # noqa: E402

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "sml_cases.npz"))


def _rk4(d_t, **kw):
    return fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), d_t, **kw)


@pytest.mark.parametrize("batched", [True, False])
@pytest.mark.parametrize("name", sorted(SML_CASES))
def test_generate_data_with_the_gpu_oracle_matches_the_reference(name, batched):
    builder, kw, op_kw, gen_kw = SML_CASES[name]
    ivp = getattr(problems, builder)(ns, **kw)
    op = SupervisedMLOperator(SML_D_T, **op_kw)
    x, y = op.generate_data(ivp, _rk4(SML_ORACLE_D_T), perturbation_function=problems.sml_perturbation,
                            batched=batched, **gen_kw)
    want_x, want_y = GOLD[f"{name}_x"], GOLD[f"{name}_y"]
    assert x.shape == want_x.shape and y.shape == want_y.shape
    assert np.allclose(x, want_x, rtol=1e-12, atol=1e-14)
    assert np.allclose(y, want_y, rtol=1e-12, atol=1e-14)


def test_chains_batched_across_iterations():
    """batch_iterations: the chained auto-regressive data of all iterations
    advanced together; with a perturbation that draws no random numbers
    the data equal the one-chain-at-a-time generation."""
    ivp = problems.diffusion_2d(ns, n=10, t_end=0.2)

    def bump(t, y):
        return y * (1.0 + 0.01 * np.cos(y + t))

    op = SupervisedMLOperator(SML_D_T, True)
    a = op.generate_data(ivp, _rk4(SML_ORACLE_D_T), 3, bump, batched=False)
    b = op.generate_data(ivp, _rk4(SML_ORACLE_D_T), 3, bump, batch_iterations=True)
    assert np.allclose(a[0], b[0], rtol=1e-13, atol=0) and np.allclose(a[1], b[1], rtol=1e-13, atol=0)


def _cnn_setup():
    ivp = problems.cahn_hilliard_2d(ns, n=24, length=6.0, t_end=0.08)
    cp = ivp.constrained_problem
    op = SupervisedMLOperator(0.01, True)
    oracle = _rk4(0.001, dtype="float32")
    np.random.seed(0)
    data = op.generate_data(ivp, oracle, 6, lambda t, y: y + 0.02 * np.random.standard_normal(y.shape),
                            isolate_perturbations=True, layout="fields")
    base = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.0025,
                           dtype="float32")
    return ivp, cp, op, data, base


def test_cnn_regressor_behind_the_model_contract():
    """The CNN regressor fits the generated states (the training loss falls),
    ``predict`` on the reference's rows equals ``predict_fields`` on the
    states, and the operator's device roll-out equals the reference's
    row-by-row auto-regressive loop through ``predict``."""
    ivp, cp, op, data, base = _cnn_setup()
    x, y = data
    assert x.shape == (48, 25, 25, 2)
    model = CNNRegressor(cp, 0.01, base=base, epochs=25, batch=8, lr=2e-3)
    train, test = op.fit_model(model, data, test_size=0.25)
    assert model.history[-1] < model.history[0]
    assert np.isfinite(train) and np.isfinite(test)
    rows = np.zeros((2 * 625, 2 * 625 + 2))
    rows[:625, :1250] = x[0].reshape(1, -1)
    rows[625:, :1250] = x[1].reshape(1, -1)
    assert np.array_equal(model.predict(rows), model.predict_fields(x[:2]).reshape(-1, 2))
    fast = op.solve(ivp).discrete_y()

    class RowsOnly:
        def predict(self, inputs):
            return model.predict(inputs)

    slow_op = SupervisedMLOperator(0.01, True)
    slow_op.model = RowsOnly()
    slow = slow_op.solve(ivp).discrete_y()
    assert fast.shape == slow.shape == (8, 25, 25, 2)
    assert np.array_equal(fast, slow)


def test_learned_operator_as_parareal_coarse_operator():
    """The supervised operator with the CNN regressor serves as Parareal's
    coarse operator (device propagation); with as many iterations as
    slices Parareal returns the fine solution."""
    ivp, cp, op, data, base = _cnn_setup()
    op.fit_model(CNNRegressor(cp, 0.01, base=base, epochs=10, batch=8), data, test_size=0.0)
    f = _rk4(0.001, dtype="float32")
    par = PararealOperator(f, op, 0.0, 4, n_slices=4, trajectory="final")
    got = par.solve(ivp).discrete_y()[-1]
    want = f.solve(ivp).discrete_y()[-1]
    assert rel_l2(got, want) < 1e-6
