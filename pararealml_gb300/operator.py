"""The operator contract (the drop-in boundary).

Same contract as ``pararealml/operator.py:13-74``: an ``Operator`` has a time
step ``d_t`` (must be positive), a ``vertex_oriented`` flag and
``solve(ivp, parallel_enabled=True) -> Solution``; the time grid is
``t0 + k*d_t`` for ``k = 0..round((t1 - t0)/d_t)`` built with ``linspace``.
"""

from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Optional

import numpy as np

from .initial_value_problem import InitialValueProblem, TemporalDomainInterval
from .solution import Solution


class Operator(ABC):
    def __init__(self, d_t: float, vertex_oriented: Optional[bool]):
        if d_t <= 0.0:
            raise ValueError("time step size must be greater than 0")
        self._d_t = d_t
        self._vertex_oriented = vertex_oriented

    d_t = property(lambda self: self._d_t)
    vertex_oriented = property(lambda self: self._vertex_oriented)

    @abstractmethod
    def solve(self, ivp: InitialValueProblem, parallel_enabled: bool = True) -> Solution:
        """Returns the IVP's solution."""


def discretize_time_domain(t: TemporalDomainInterval, d_t: float) -> np.ndarray:
    t_0 = t[0]
    steps = int(round((t[1] - t_0) / d_t))
    return np.linspace(t_0, t_0 + steps * d_t, steps + 1)
