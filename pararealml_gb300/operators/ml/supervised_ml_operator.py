"""Supervised learned operator with the reference's API.

Mirrors ``SupervisedMLOperator``
(``pararealml/operators/ml/supervised/supervised_ml_operator.py``): an
``Operator`` with its own ``d_t`` whose regression model (anything with
scikit-learn's ``fit(x, y)`` / ``predict(x)``) maps the solution at one time
point to the next, trained on data an oracle operator generates from
perturbed initial conditions.  The model inputs, the data generation
(perturbation order, auto-regression, isolated perturbations, jobs and their
seeds), the random train / test split and the auto-regressive ``solve`` follow
the reference's semantics, so that with the same oracle results, model and
seeds both produce the same arrays.

GB300 additions, all keyword-only:

* The oracle's sub-IVP solves run on the GPU.  When the oracle is this
  package's ``FDMOperator`` and the order in which the perturbation function
  is called does not depend on solve results (non-auto-regressive
  generation, or isolated perturbations), all perturbed initial states of a
  job are drawn first, in the reference's order, and advanced in ONE
  batched device solve (``batched=True``, the default; problems with
  time-dependent boundary conditions, time-dependent right-hand sides or
  Jacobi rows, and ``repeat_on_error``, take the one-solve-per-sub-IVP path).
  ``batch_iterations=True`` also batches chained auto-regressive generation
  across iterations, calling the perturbation function time step by time
  step instead of iteration by iteration (identical data for a perturbation
  that draws no random numbers).
* ``layout="fields"`` returns (and ``fit_model`` accepts) the data as states:
  inputs and targets of shape (N, *vertices, y_dim), one pair per sub-IVP,
  instead of the reference's rows of [all y values, t or d_t, x] per vertex,
  whose size grows with the square of the mesh (about 70 GB per time point
  on a 257^2 mesh with 2 components).  A model with ``predict_fields``
  (``learned.CNNRegressor``) is applied to whole states by ``solve``.
"""

from __future__ import annotations

import math
import warnings
from typing import Any, Callable, List, Optional, Sequence, Tuple

import numpy as np

from ...initial_condition import DiscreteInitialCondition
from ...initial_value_problem import InitialValueProblem
from ...operator import Operator, discretize_time_domain
from ...solution import Solution


def mean_squared_error(y_true: np.ndarray, y_pred: np.ndarray) -> float:
    """The mean over outputs of each output's mean squared error
    (scikit-learn's ``mean_squared_error`` with uniform output weights, the
    reference's default score)."""
    y_true = np.asarray(y_true, dtype=float)
    y_pred = np.asarray(y_pred, dtype=float)
    if y_true.ndim == 1:
        y_true = y_true.reshape(-1, 1)
        y_pred = y_pred.reshape(-1, 1)
    return float(np.average(np.average((y_true - y_pred) ** 2, axis=0)))


def train_test_indices(n: int, test_size: float) -> Tuple[np.ndarray, np.ndarray]:
    """Random (train, test) indices as scikit-learn's ``train_test_split``
    draws them without a random state: ceil(test_size n) test samples, the
    rest for training, from one permutation of numpy's global generator
    (test first)."""
    n_test = int(math.ceil(test_size * n))
    n_train = n - n_test
    if n_train <= 0 or n_test <= 0:
        raise ValueError(f"test_size {test_size} leaves an empty train or test set for {n} samples")
    perm = np.random.permutation(n)
    return perm[n_test:n_test + n_train], perm[:n_test]


def _autonomous(cp) -> bool:
    """Whether sub-IVP solves are independent of their start times: static
    boundary conditions, right-hand sides without t, and no Jacobi rows
    (whose initial estimates come from numpy's global generator)."""
    from ...differential_equation import LHS

    if not cp.are_all_boundary_conditions_static:
        return False
    system = cp.differential_equation.symbolic_equation_system
    if any(lhs == LHS.Y_LAPLACIAN for lhs in system.lhs_types):
        return False
    return not any(sym.name == "t" for expr in system.rhs for sym in expr.free_symbols)


class SupervisedMLOperator(Operator):
    """A supervised machine learning operator that models a high fidelity
    operator for solving initial value problems (supervised_ml_operator.py:
    16-128): ``auto_regressive`` feeds each prediction back as the next
    input, ``time_variant`` adds the time as a predictor, ``input_d_t`` adds
    the operator's time step."""

    def __init__(self, d_t: float, vertex_oriented: bool, auto_regressive: bool = True,
                 time_variant: bool = False, input_d_t: bool = False):
        if not auto_regressive and not time_variant:
            raise ValueError("operator must be time variant if auto-regression is disabled")
        if time_variant and input_d_t:
            raise ValueError("operator must be time invariant to use d_t as an input")
        super().__init__(d_t, vertex_oriented)
        self._auto_regressive = auto_regressive
        self._time_variant = time_variant
        self._input_d_t = input_d_t
        self._model: Optional[Any] = None

    auto_regressive = property(lambda self: self._auto_regressive)
    time_variant = property(lambda self: self._time_variant)
    input_d_t = property(lambda self: self._input_d_t)

    @property
    def model(self) -> Optional[Any]:
        return self._model

    @model.setter
    def model(self, model: Optional[Any]):
        self._model = model

    # ------------------------------------------------------------------ solve
    def solve(self, ivp: InitialValueProblem, parallel_enabled: bool = True) -> Solution:
        """The model applied step by step (supervised_ml_operator.py:91-128):
        the inputs of each step are the previous output (auto-regressive) or
        the initial state, plus t or d_t, plus the coordinates."""
        if self._model is None:
            raise ValueError("operator has no model")
        cp = ivp.constrained_problem
        diff_eq = cp.differential_equation
        y_shape = cp.y_shape(self._vertex_oriented)
        t = discretize_time_domain(ivp.t_interval, self._d_t)[1:]
        y_0 = ivp.initial_condition.discrete_y_0(self._vertex_oriented)
        if (hasattr(self._model, "predict_fields") and self._auto_regressive and not self._time_variant
                and not self._input_d_t):
            # a state-to-state model: every step on whole device states
            y = self._model.rollout(y_0, len(t))
            return Solution(ivp, t, y, vertex_oriented=self._vertex_oriented, d_t=self._d_t)
        inputs = self._create_input_placeholder(cp)
        y = np.empty((len(t),) + y_shape)
        n_y = inputs.shape[1] - diff_eq.x_dimension - (self._time_variant or self._input_d_t)
        for i, t_i in enumerate(t):
            inputs[:, :n_y] = y_0.reshape((1, -1))
            if self._time_variant:
                inputs[:, -diff_eq.x_dimension - 1] = t_i
            elif self._input_d_t:
                inputs[:, -diff_eq.x_dimension - 1] = self._d_t
            y_i = self._model.predict(inputs)
            y[i, ...] = y_i.reshape(y_shape)
            if self._auto_regressive:
                y_0 = y_i
        return Solution(ivp, t, y, vertex_oriented=self._vertex_oriented, d_t=self._d_t)

    def coarse_propagator(self, cp, batch: int, n_steps: int):
        """Parareal's coarse sweep on device states, for a model that
        provides one (``learned.CNNRegressor``, auto-regressive and
        time-invariant); other models run through ``solve`` only."""
        if (self._model is None or not hasattr(self._model, "coarse_propagator") or not self._auto_regressive
                or self._time_variant or self._input_d_t):
            raise NotImplementedError("the model has no device propagation")
        return self._model.coarse_propagator(cp, batch, n_steps)

    # -------------------------------------------------------- data generation
    def generate_data(self, ivp: InitialValueProblem, oracle: Operator, iterations: int,
                      perturbation_function: Callable[[float, np.ndarray], np.ndarray],
                      isolate_perturbations: bool = False, repeat_on_error: bool = False, n_jobs: int = 1,
                      seeds: Optional[Sequence[int]] = None, *, layout: str = "rows", batched: bool = True,
                      batch_iterations: bool = False) -> Tuple[np.ndarray, np.ndarray]:
        """Inputs and targets from the oracle's solutions of sub-IVPs with
        perturbed initial conditions (supervised_ml_operator.py:130-236).
        ``iterations`` are split into ``n_jobs`` contiguous chunks, chunk r
        generated after ``np.random.seed(seeds[r])`` (when seeds are given)
        and the chunks concatenated in order, as the reference's processes
        do; here the chunks run one after another on the GPU."""
        if iterations <= 0:
            raise ValueError("number of iterations must be greater than 0")
        if n_jobs < 1:
            raise ValueError("number of jobs must be greater than 0")
        if seeds is not None:
            if len(seeds) != n_jobs:
                raise ValueError(f"number of seeds ({len(seeds)}) must match number of jobs ({n_jobs})")
        else:
            seeds = [None] * n_jobs
        if layout not in ("rows", "fields"):
            raise ValueError("layout must be 'rows' or 'fields'")
        chunks = np.array_split(np.arange(iterations), n_jobs) if n_jobs > 1 else [np.arange(iterations)]
        parts = [
            self._generate_chunk(ivp, oracle, len(idx), perturbation_function, isolate_perturbations,
                                 repeat_on_error, seeds[rank], layout, batched, batch_iterations)
            for rank, idx in enumerate(chunks)
        ]
        return np.concatenate([p[0] for p in parts], axis=0), np.concatenate([p[1] for p in parts], axis=0)

    def fit_model(self, model: Any, data: Tuple[np.ndarray, np.ndarray], test_size: float = 0.2,
                  score_func: Callable[[np.ndarray, np.ndarray], float] = mean_squared_error
                  ) -> Tuple[float, Optional[float]]:
        """Fits the model to a random training share of the data and keeps
        it (supervised_ml_operator.py:238-284): the split is scikit-learn's
        (``train_test_indices``), or one permutation of all data without a
        test share; returns the training and test scores."""
        x, y = data
        if test_size:
            train, test = train_test_indices(len(x), test_size)
            x_train, x_test, y_train, y_test = x[train], x[test], y[train], y[test]
        else:
            shuffled = np.random.permutation(len(x))
            x_train, y_train = x[shuffled], y[shuffled]
            x_test = y_test = None
        model.fit(x_train, y_train)
        self._model = model
        train_score = score_func(y_train, self._predict_data(model, x_train))
        test_score = score_func(y_test, self._predict_data(model, x_test)) if test_size else None
        return train_score, test_score

    def train(self, ivp: InitialValueProblem, oracle: Operator, model: Any, iterations: int,
              perturbation_function: Callable[[float, np.ndarray], np.ndarray], isolate_perturbations: bool = False,
              repeat_on_error: bool = False, n_jobs: int = 1, seeds: Optional[Sequence[int]] = None,
              test_size: float = 0.2, score_func: Callable[[np.ndarray, np.ndarray], float] = mean_squared_error,
              **gb300) -> Tuple[float, Optional[float]]:
        """``generate_data`` then ``fit_model`` (supervised_ml_operator.py:286-357)."""
        data = self.generate_data(ivp, oracle, iterations, perturbation_function,
                                  isolate_perturbations=isolate_perturbations, repeat_on_error=repeat_on_error,
                                  n_jobs=n_jobs, seeds=seeds, **gb300)
        return self.fit_model(model, data, test_size=test_size, score_func=score_func)

    # ---------------------------------------------------------------- helpers
    @staticmethod
    def _predict_data(model, x):
        if x.ndim > 2 and hasattr(model, "predict_fields"):
            return model.predict_fields(x)
        return model.predict(x)

    def _create_input_placeholder(self, cp) -> np.ndarray:
        """One row per spatial point: [y at every point, (t or d_t), x]
        (supervised_ml_operator.py:359-382); an ODE has one row [y, (t)]."""
        diff_eq = cp.differential_equation
        if not diff_eq.x_dimension:
            return np.empty((1, diff_eq.y_dimension + self._time_variant))
        x = cp.mesh.all_index_coordinates(self._vertex_oriented, flatten=True)
        y = np.empty((len(x), diff_eq.y_dimension * len(x)))
        if self._time_variant or self._input_d_t:
            return np.hstack([y, np.empty((len(x), 1)), x])
        return np.hstack([y, x])

    def _perturb(self, t0: float, y_0: np.ndarray, cp, perturbation_function) -> np.ndarray:
        perturbed = perturbation_function(t0, y_0)
        if perturbed.shape != y_0.shape:
            raise ValueError(f"perturbed y shape {perturbed.shape} must match input y shape {y_0.shape}")
        return perturbed

    def _perturb_and_solve_ivp(self, ivp: InitialValueProblem, perturbation_function, oracle: Operator,
                               repeat_on_error: bool) -> Solution:
        """Perturbs the IVP's initial state and solves it with the oracle,
        perturbing anew after a failed solve when ``repeat_on_error``
        (supervised_ml_operator.py:527-578)."""
        while True:
            y_0 = ivp.initial_condition.discrete_y_0(self._vertex_oriented)
            perturbed_y_0 = self._perturb(ivp.t_interval[0], y_0, ivp.constrained_problem, perturbation_function)
            perturbed_ivp = InitialValueProblem(
                ivp.constrained_problem, ivp.t_interval,
                DiscreteInitialCondition(ivp.constrained_problem, perturbed_y_0, self._vertex_oriented))
            try:
                return oracle.solve(perturbed_ivp)
            except Exception as exception:  # the reference's contract: any solve failure
                if repeat_on_error:
                    warnings.warn(f"Failed to solve IVP with perturbed initial conditions; {str(exception)}")
                    continue
                raise exception

    def _batched_solver(self, cp, oracle, batched: bool, repeat_on_error: bool):
        """A device solver of many sub-IVPs of this operator's d_t at once,
        or None when the oracle or the problem needs one solve per sub-IVP."""
        from ..fdm.fdm_operator import FDMOperator

        if not (batched and not repeat_on_error and isinstance(oracle, FDMOperator) and self._vertex_oriented
                and _autonomous(cp)):
            return None
        per = int(round(self._d_t / oracle.d_t))
        if per < 1 or not np.isclose(per * oracle.d_t, self._d_t, rtol=1e-12, atol=0.0):
            return None

        def solve(y0s: np.ndarray, t0: float, n_out: int) -> np.ndarray:
            """(N, *vertices, C) states -> the states after 1..n_out steps of
            d_t: (n_out, N, *vertices, C)."""
            import torch

            plan = oracle.plan(cp, y0s.shape[0])
            dev = torch.from_numpy(np.ascontiguousarray(y0s, dtype=np.float64)).to(plan.device)
            traj = oracle.solve_device(cp, dev, float(t0), n_out * per, save_every=per)
            plan.check_status()
            out = plan.unpack(traj, n_out * y0s.shape[0]).cpu().numpy()
            return out.reshape((n_out, y0s.shape[0]) + tuple(y0s.shape[1:]))

        return solve

    def _generate_chunk(self, ivp, oracle, iterations, perturbation_function, isolate_perturbations,
                        repeat_on_error, seed, layout, batched, batch_iterations):
        """One job's data (supervised_ml_operator.py:384-525)."""
        if seed is not None:
            np.random.seed(seed)
        cp = ivp.constrained_problem
        diff_eq = cp.differential_equation
        x_dim, y_dim = diff_eq.x_dimension, diff_eq.y_dimension
        vo = self._vertex_oriented
        t = discretize_time_domain(ivp.t_interval, self._d_t)
        n_t = len(t) - 1
        y_0 = ivp.initial_condition.discrete_y_0(vo)
        solver = self._batched_solver(cp, oracle, batched, repeat_on_error)

        unperturbed: Optional[np.ndarray] = None
        if self._auto_regressive and isolate_perturbations:
            unperturbed = self._perturb_and_solve_ivp(
                InitialValueProblem(cp, (t[0], t[-2]), ivp.initial_condition), lambda _, y: y, oracle, False,
            ).discrete_y(vo)[np.rint((t[1:-1] - t[0]) / oracle.d_t).astype(int) - 1, ...]

        # (iteration, time step) -> perturbed input state and target state
        ins: List[List[Optional[np.ndarray]]] = [[None] * n_t for _ in range(iterations)]
        outs: List[List[Optional[np.ndarray]]] = [[None] * n_t for _ in range(iterations)]

        def constrained(y):
            return DiscreteInitialCondition(cp, y, vo).discrete_y_0(vo)

        if self._auto_regressive:
            if solver is not None and isolate_perturbations:
                # the inputs do not depend on any perturbed solve: draw every
                # perturbation in the reference's order, then one solve
                for it in range(iterations):
                    for i in range(n_t):
                        y_i = constrained(y_0 if i == 0 else unperturbed[i - 1])
                        ins[it][i] = constrained(self._perturb(t[i], y_i, cp, perturbation_function))
                flat = np.stack([ins[it][i] for it in range(iterations) for i in range(n_t)])
                res = solver(flat, float(t[0]), 1)[0]
                for k, (it, i) in enumerate((it, i) for it in range(iterations) for i in range(n_t)):
                    outs[it][i] = res[k]
            elif solver is not None and batch_iterations:
                # chains advanced together, time step by time step
                y_i = [y_0] * iterations
                for i in range(n_t):
                    for it in range(iterations):
                        src = constrained(y_i[it])
                        ins[it][i] = constrained(self._perturb(t[i], src, cp, perturbation_function))
                    res = solver(np.stack([ins[it][i] for it in range(iterations)]), float(t[i]), 1)[0]
                    for it in range(iterations):
                        outs[it][i] = res[it]
                        y_i[it] = (unperturbed[i] if isolate_perturbations and i < n_t - 1 else res[it])
            else:
                for it in range(iterations):
                    y_i = y_0
                    for i, t_i in enumerate(t[:-1]):
                        sol = self._perturb_and_solve_ivp(
                            InitialValueProblem(cp, (t_i, t_i + self._d_t), DiscreteInitialCondition(cp, y_i, vo)),
                            perturbation_function, oracle, repeat_on_error)
                        ins[it][i] = sol.initial_value_problem.initial_condition.discrete_y_0(vo)
                        outs[it][i] = sol.discrete_y(vo)[-1]
                        y_i = unperturbed[i] if isolate_perturbations and i < n_t - 1 else outs[it][i]
        else:
            if solver is not None:
                firsts = [constrained(self._perturb(ivp.t_interval[0], y_0, cp, perturbation_function))
                          for _ in range(iterations)]
                res = solver(np.stack(firsts), float(t[0]), n_t)
                for it in range(iterations):
                    for i in range(n_t):
                        ins[it][i], outs[it][i] = firsts[it], res[i, it]
            else:
                for it in range(iterations):
                    sol = self._perturb_and_solve_ivp(ivp, perturbation_function, oracle, repeat_on_error)
                    first = sol.initial_value_problem.initial_condition.discrete_y_0(vo)
                    y = sol.discrete_y(vo)[np.rint((t[1:] - t[0]) / oracle.d_t).astype(int) - 1, ...]
                    for i in range(n_t):
                        ins[it][i], outs[it][i] = first, y[i]

        if layout == "fields":
            return (np.stack([ins[it][i] for it in range(iterations) for i in range(n_t)]),
                    np.stack([outs[it][i] for it in range(iterations) for i in range(n_t)]))
        single = self._create_input_placeholder(cp)
        n_pts = single.shape[0]
        epoch = np.tile(single, (n_t, 1))
        if self._time_variant:
            epoch[:, -x_dim - 1] = np.repeat(t[1:], n_pts)
        elif self._input_d_t:
            epoch[:, -x_dim - 1] = self._d_t
        inputs = np.tile(epoch, (iterations, 1))
        targets = np.empty((inputs.shape[0], y_dim))
        n_y = inputs.shape[1] - x_dim - (self._time_variant if not self._auto_regressive else 0)
        for it in range(iterations):
            offset = it * n_pts * n_t
            for i in range(n_t):
                rows = slice(offset + i * n_pts, offset + (i + 1) * n_pts)
                if self._auto_regressive:
                    inputs[rows, :y_dim * n_pts] = ins[it][i].reshape((1, -1))
                else:
                    inputs[rows, :n_y] = ins[it][i].reshape((1, -1))
                targets[rows, :] = outs[it][i].reshape((-1, y_dim))
        return inputs, targets
