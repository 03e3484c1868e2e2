"""Initial value problems (host side); same surface as
``pararealml/initial_value_problem.py:13-92``."""

from __future__ import annotations

from typing import Callable, Optional, Tuple

import numpy as np

from .constrained_problem import ConstrainedProblem
from .initial_condition import InitialCondition

TemporalDomainInterval = Tuple[float, float]


class InitialValueProblem:
    def __init__(
        self,
        cp: ConstrainedProblem,
        t_interval: TemporalDomainInterval,
        initial_condition: InitialCondition,
        exact_y: Optional[Callable[["InitialValueProblem", float, Optional[np.ndarray]], np.ndarray]] = None,
    ):
        if t_interval[0] > t_interval[1]:
            raise ValueError(
                f"lower bound of time interval ({t_interval[0]}) cannot be "
                f"greater than its upper bound ({t_interval[1]})"
            )
        self._cp = cp
        self._t_interval = t_interval
        self._initial_condition = initial_condition
        self._exact_y = exact_y

    constrained_problem = property(lambda self: self._cp)
    t_interval = property(lambda self: self._t_interval)
    initial_condition = property(lambda self: self._initial_condition)
    has_exact_solution = property(lambda self: self._exact_y is not None)

    def exact_y(self, t: float, x: Optional[np.ndarray] = None) -> np.ndarray:
        if not self.has_exact_solution:
            raise RuntimeError("exact solution of initial value problem undefined")
        return self._exact_y(self, t, x)
