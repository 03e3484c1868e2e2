"""Boundary conditions (host side).

Same classes and flags as ``pararealml/boundary_condition.py:11-287``.  A
condition function maps ``(x: (n, x_dim), t)`` to an ``(n, y_dim)`` array in
which NaN means "this component is not constrained at this point".  The GPU
path evaluates these functions once on the host (static conditions) and
uploads the resulting face tables.
"""

from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Callable, Optional, Sequence

import numpy as np

VectorizedBoundaryConditionFunction = Callable[[np.ndarray, Optional[float]], np.ndarray]


class BoundaryCondition(ABC):
    def __init__(self, has_y_condition: bool, has_d_y_condition: bool, is_static: bool):
        self._has_y_condition = has_y_condition
        self._has_d_y_condition = has_d_y_condition
        self._is_static = is_static

    has_y_condition = property(lambda self: self._has_y_condition)
    has_d_y_condition = property(lambda self: self._has_d_y_condition)
    is_static = property(lambda self: self._is_static)

    @abstractmethod
    def y_condition(self, x: np.ndarray, t: Optional[float]) -> np.ndarray:
        """Values of y on the boundary points ``x`` (NaN = unconstrained)."""

    @abstractmethod
    def d_y_condition(self, x: np.ndarray, t: Optional[float]) -> np.ndarray:
        """Values of the outward... normal derivative of y (NaN = unconstrained)."""


class DirichletBoundaryCondition(BoundaryCondition):
    def __init__(self, y_condition: VectorizedBoundaryConditionFunction, is_static: bool = False):
        super().__init__(True, False, is_static)
        self._y_condition = y_condition

    def y_condition(self, x, t):
        return self._y_condition(x, t)

    def d_y_condition(self, x, t):
        raise RuntimeError("Dirichlet conditions do not constrain the derivative of y")


class NeumannBoundaryCondition(BoundaryCondition):
    def __init__(
        self, d_y_condition: VectorizedBoundaryConditionFunction, is_static: bool = False
    ):
        super().__init__(False, True, is_static)
        self._d_y_condition = d_y_condition

    def y_condition(self, x, t):
        raise RuntimeError("Neumann conditions do not constrain the value of y")

    def d_y_condition(self, x, t):
        return self._d_y_condition(x, t)


class CauchyBoundaryCondition(BoundaryCondition):
    def __init__(
        self,
        y_condition: VectorizedBoundaryConditionFunction,
        d_y_condition: VectorizedBoundaryConditionFunction,
        is_static: bool = False,
    ):
        super().__init__(True, True, is_static)
        self._y_condition = y_condition
        self._d_y_condition = d_y_condition

    def y_condition(self, x, t):
        return self._y_condition(x, t)

    def d_y_condition(self, x, t):
        return self._d_y_condition(x, t)


class ConstantBoundaryCondition(BoundaryCondition):
    """Space- and time-independent conditions; ``None`` entries are unconstrained."""

    def __init__(
        self,
        constant_y_conditions: Optional[Sequence[Optional[float]]],
        constant_d_y_conditions: Optional[Sequence[Optional[float]]],
    ):
        if constant_y_conditions is None and constant_d_y_conditions is None:
            raise ValueError("at least one type of constant conditions must not be None")
        self._y_const = constant_y_conditions
        self._d_y_const = constant_d_y_conditions
        super().__init__(
            constant_y_conditions is not None, constant_d_y_conditions is not None, True
        )

    @staticmethod
    def _fill(values, n):
        return np.array(
            [[np.nan if v is None else float(v) for v in values]] * n, dtype=float
        ).reshape((n, len(values)))

    def y_condition(self, x, t):
        if not self._y_const:
            raise RuntimeError("no boundary conditions defined on y")
        return self._fill(self._y_const, len(x))

    def d_y_condition(self, x, t):
        if not self._d_y_const:
            raise RuntimeError("no boundary conditions defined on the normal derivative of y")
        return self._fill(self._d_y_const, len(x))


class ConstantValueBoundaryCondition(ConstantBoundaryCondition):
    def __init__(self, constant_y_conditions: Sequence[Optional[float]]):
        super().__init__(constant_y_conditions, None)


class ConstantFluxBoundaryCondition(ConstantBoundaryCondition):
    def __init__(self, constant_d_y_conditions: Sequence[Optional[float]]):
        super().__init__(None, constant_d_y_conditions)


def vectorize_bc_function(
    bc_function: Callable[[Sequence[float], Optional[float]], Sequence[Optional[float]]]
) -> VectorizedBoundaryConditionFunction:
    """Lifts a per-point condition function to an ``(n, x_dim)`` -> ``(n, y_dim)`` one."""

    def vectorized(x: np.ndarray, t: Optional[float]) -> np.ndarray:
        return np.array([bc_function(x[i], t) for i in range(len(x))], dtype=float)

    return vectorized
