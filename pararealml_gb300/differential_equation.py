"""Symbolic differential equations (host side).

Mirrors the public surface of ``pararealml/differential_equation.py`` so that
problems written against the reference construct unchanged here:
``Symbols`` (``:10-139``), ``LHS`` (``:142-150``), ``SymbolicEquationSystem``
(``:153-211``), ``DifferentialEquation`` (``:214-352``) and the PDEs whose
right-hand sides the GPU code generator lowers (Diffusion ``:608-630``,
ConvectionDiffusion ``:633-667``, Wave ``:670-697``, Cahn-Hilliard
``:700-731``, Burgers ``:734-765``, ShallowWater ``:768-819``,
NavierStokes ``:822-850``).

Symbol names follow the reference grammar exactly (``y_i``, ``x_j``,
``y-gradient_i_j``, ``y-hessian_i_j_k``, ``y-laplacian_i``,
``y-divergence_i_j..``, ``y-curl_..``, ``y-vector-laplacian_..``) because the
code generator parses them by name.
"""

from __future__ import annotations

from abc import ABC, abstractmethod
from copy import copy, deepcopy
from enum import Enum
from typing import Dict, List, Optional, Sequence, Union

import numpy as np
from sympy import Expr, Symbol, symarray


class Symbols:
    """The symbols a differential equation of a given size may use."""

    def __init__(self, x_dimension: int, y_dimension: int):
        self._t = Symbol("t")
        self._y = symarray("y", (y_dimension,))
        self._x = self._y_gradient = self._y_hessian = None
        self._y_divergence = self._y_curl = None
        self._y_laplacian = self._y_vector_laplacian = None
        if x_dimension:
            self._x = symarray("x", (x_dimension,))
            self._y_gradient = symarray("y-gradient", (y_dimension, x_dimension))
            self._y_hessian = symarray(
                "y-hessian", (y_dimension, x_dimension, x_dimension)
            )
            self._y_divergence = symarray("y-divergence", (y_dimension,) * x_dimension)
            if 2 <= x_dimension <= 3:
                curl_shape = (
                    ((y_dimension,) * x_dimension) + (x_dimension,)
                    if x_dimension == 3
                    else ()
                )
                self._y_curl = symarray("y-curl", curl_shape)
            self._y_laplacian = symarray("y-laplacian", (y_dimension,))
            self._y_vector_laplacian = symarray(
                "y-vector-laplacian", ((y_dimension,) * x_dimension) + (x_dimension,)
            )

    t = property(lambda self: self._t)
    y = property(lambda self: copy(self._y))
    x = property(lambda self: copy(self._x))
    y_gradient = property(lambda self: copy(self._y_gradient))
    y_hessian = property(lambda self: copy(self._y_hessian))
    y_divergence = property(lambda self: copy(self._y_divergence))
    y_curl = property(lambda self: copy(self._y_curl))
    y_laplacian = property(lambda self: copy(self._y_laplacian))
    y_vector_laplacian = property(lambda self: copy(self._y_vector_laplacian))


class LHS(Enum):
    """Left-hand side kinds of the equations of a system."""

    D_Y_OVER_D_T = 0
    Y = 1
    Y_LAPLACIAN = 2


class SymbolicEquationSystem:
    """Right-hand sides plus their left-hand side kinds."""

    def __init__(
        self,
        rhs: Union[Sequence[Expr], np.ndarray],
        lhs_types: Optional[Sequence[LHS]] = None,
    ):
        if len(rhs) < 1:
            raise ValueError("number of equations must be greater than 0")
        if lhs_types is None:
            lhs_types = [LHS.D_Y_OVER_D_T] * len(rhs)
        if len(rhs) != len(lhs_types):
            raise ValueError(
                f"length of right-hand side ({len(rhs)}) must match length of "
                f"left-hand side ({len(lhs_types)})"
            )
        self._rhs = copy(rhs)
        self._lhs_types = copy(lhs_types)
        self._by_type: Dict[LHS, List[int]] = {k: [] for k in LHS}
        for i, kind in enumerate(lhs_types):
            self._by_type[kind].append(i)

    @property
    def rhs(self):
        return copy(self._rhs)

    @property
    def lhs_types(self) -> Sequence[LHS]:
        return copy(self._lhs_types)

    def equation_indices_by_type(self, lhs_type: LHS) -> Sequence[int]:
        return copy(self._by_type[lhs_type])


class DifferentialEquation(ABC):
    """A time-dependent differential equation (ODE if ``x_dimension == 0``)."""

    def __init__(
        self,
        x_dimension: int,
        y_dimension: int,
        all_vector_field_indices: Optional[Sequence[Sequence[int]]] = None,
    ):
        if x_dimension < 0:
            raise ValueError(
                f"number of x dimensions ({x_dimension}) must be non-negative"
            )
        if y_dimension < 1:
            raise ValueError(
                f"number of y dimensions ({y_dimension}) must be at least 1"
            )
        for indices in all_vector_field_indices or []:
            if len(indices) != x_dimension:
                raise ValueError(
                    f"length of vector field indices {indices} must match "
                    f"x dimensions ({x_dimension})"
                )
            if any(not (0 <= i < y_dimension) for i in indices):
                raise ValueError(
                    "all indices must be non-negative and less than "
                    f"the number of y dimensions ({y_dimension})"
                )
        self._x_dimension = x_dimension
        self._y_dimension = y_dimension
        self._all_vector_field_indices = deepcopy(all_vector_field_indices)
        self._symbols = Symbols(x_dimension, y_dimension)
        self._validate_equations()

    x_dimension = property(lambda self: self._x_dimension)
    y_dimension = property(lambda self: self._y_dimension)
    symbols = property(lambda self: self._symbols)
    all_vector_field_indices = property(
        lambda self: deepcopy(self._all_vector_field_indices)
    )

    @property
    @abstractmethod
    def symbolic_equation_system(self) -> SymbolicEquationSystem:
        """The system of symbolic equations defining the equation."""

    def _validate_equations(self):
        eq_sys = self.symbolic_equation_system
        if len(eq_sys.rhs) != self._y_dimension:
            raise ValueError(
                f"number of equations ({len(eq_sys.rhs)}) must match "
                f"number of y dimensions ({self._y_dimension})"
            )
        s = self._symbols
        allowed = {s.t, *s.y}
        if self._x_dimension:
            allowed.update(s.x)
            allowed.update(s.y_gradient.flatten())
            allowed.update(s.y_hessian.flatten())
            allowed.update(s.y_divergence.flatten())
            if 2 <= self._x_dimension <= 3:
                allowed.update(s.y_curl.flatten())
            allowed.update(s.y_laplacian)
            allowed.update(s.y_vector_laplacian.flatten())
        for i, rhs in enumerate(eq_sys.rhs):
            if not rhs.free_symbols.issubset(allowed):
                raise ValueError(
                    "invalid symbol in right-hand side symbols "
                    f"({rhs.free_symbols}) of equation {i}"
                )
        n_dt = len(eq_sys.equation_indices_by_type(LHS.D_Y_OVER_D_T))
        if self._x_dimension:
            if n_dt == 0:
                raise ValueError(
                    "at least one equation's left-hand side must be of type "
                    "D_Y_OVER_D_T"
                )
        elif n_dt != self._y_dimension:
            raise ValueError(
                "ordinary differential equation systems can only contain "
                "equations with D_Y_OVER_D_T type left-hand sides"
            )


def _require_pde(x_dimension: int):
    if x_dimension <= 0:
        raise ValueError(f"number of x dimensions ({x_dimension}) must be at least 1")


class PopulationGrowthEquation(DifferentialEquation):
    """``dy/dt = r*y`` (reference ``differential_equation.py:355-377``)."""

    def __init__(self, r: float = 0.01):
        self._r = r
        super().__init__(0, 1)

    @property
    def symbolic_equation_system(self) -> SymbolicEquationSystem:
        return SymbolicEquationSystem([self._r * self._symbols.y[0]])


class DiffusionEquation(DifferentialEquation):
    """``dy/dt = d * laplacian(y)``."""

    def __init__(self, x_dimension: int, d: float = 1.0):
        _require_pde(x_dimension)
        self._d = d
        super().__init__(x_dimension, 1)

    @property
    def symbolic_equation_system(self) -> SymbolicEquationSystem:
        return SymbolicEquationSystem([self._d * self._symbols.y_laplacian[0]])


class ConvectionDiffusionEquation(DifferentialEquation):
    """``dy/dt = d * laplacian(y) - velocity . grad(y)``."""

    def __init__(self, x_dimension: int, velocity: Sequence[float], d: float = 1.0):
        _require_pde(x_dimension)
        if len(velocity) != x_dimension:
            raise ValueError(
                f"length of the velocity vector ({len(velocity)}) must match "
                f"number of x dimensions ({x_dimension})"
            )
        self._velocity = copy(velocity)
        self._d = d
        super().__init__(x_dimension, 1)

    @property
    def symbolic_equation_system(self) -> SymbolicEquationSystem:
        s = self._symbols
        return SymbolicEquationSystem(
            [self._d * s.y_laplacian[0] - np.dot(self._velocity, s.y_gradient[0, :])]
        )


class WaveEquation(DifferentialEquation):
    """Second-order wave equation as the first-order pair ``(y, dy/dt)``."""

    def __init__(self, x_dimension: int, c: float = 1.0):
        _require_pde(x_dimension)
        self._c = c
        super().__init__(x_dimension, 2)

    @property
    def symbolic_equation_system(self) -> SymbolicEquationSystem:
        s = self._symbols
        return SymbolicEquationSystem([s.y[1], (self._c**2) * s.y_laplacian[0]])


class CahnHilliardEquation(DifferentialEquation):
    """Phase separation: ``dc/dt = d*lap(mu)``, ``mu = c^3 - c - gamma*lap(c)``."""

    def __init__(self, x_dimension: int, d: float = 0.1, gamma: float = 0.01):
        _require_pde(x_dimension)
        self._d = d
        self._gamma = gamma
        super().__init__(x_dimension, 2)

    @property
    def symbolic_equation_system(self) -> SymbolicEquationSystem:
        s = self._symbols
        return SymbolicEquationSystem(
            [
                self._d * s.y_laplacian[1],
                s.y[0] ** 3 - s.y[0] - self._gamma * s.y_laplacian[0],
            ],
            [LHS.D_Y_OVER_D_T, LHS.Y],
        )


class BurgersEquation(DifferentialEquation):
    """Viscous Burgers' equations in ``x_dimension`` dimensions."""

    def __init__(self, x_dimension: int, re: float = 4000.0):
        _require_pde(x_dimension)
        self._re = re
        super().__init__(x_dimension, x_dimension, [tuple(range(x_dimension))])

    @property
    def symbolic_equation_system(self) -> SymbolicEquationSystem:
        s = self._symbols
        return SymbolicEquationSystem(
            [
                (1.0 / self._re) * s.y_laplacian[i] - np.dot(s.y, s.y_gradient[i, :])
                for i in range(self._x_dimension)
            ]
        )


class ShallowWaterEquation(DifferentialEquation):
    """Non-conservative 2D shallow water equations in ``(h, u, v)``."""

    def __init__(
        self,
        h: float,
        b: float = 0.01,
        v: float = 0.1,
        f: float = 0.0,
        g: float = 9.80665,
    ):
        self._h, self._b, self._v, self._f, self._g = h, b, v, f, g
        super().__init__(2, 3, [(1, 2)])

    @property
    def symbolic_equation_system(self) -> SymbolicEquationSystem:
        s = self._symbols
        y, grad = s.y, s.y_gradient
        return SymbolicEquationSystem(
            [
                -self._h * s.y_divergence[1, 2]
                - y[0] * grad[1, 0]
                - y[1] * grad[0, 0]
                - y[0] * grad[2, 1]
                - y[2] * grad[0, 1],
                self._v * s.y_laplacian[1]
                - y[1] * grad[1, 0]
                - y[2] * grad[1, 1]
                - self._g * grad[0, 0]
                - self._b * y[1]
                + self._f * y[2],
                self._v * s.y_laplacian[2]
                - y[1] * grad[2, 0]
                - y[2] * grad[2, 1]
                - self._g * grad[0, 1]
                - self._b * y[2]
                - self._f * y[1],
            ]
        )


class NavierStokesEquation(DifferentialEquation):
    """2D incompressible Navier-Stokes in vorticity/stream-function form."""

    def __init__(self, re: float = 4000.0):
        self._re = re
        super().__init__(2, 4, [(2, 3)])

    @property
    def symbolic_equation_system(self) -> SymbolicEquationSystem:
        s = self._symbols
        return SymbolicEquationSystem(
            [
                (1.0 / self._re) * s.y_laplacian[0]
                - np.dot(s.y[2:], s.y_gradient[0, :]),
                -s.y[0],
                s.y_gradient[1, 1],
                -s.y_gradient[1, 0],
            ],
            [LHS.D_Y_OVER_D_T, LHS.Y_LAPLACIAN, LHS.Y, LHS.Y],
        )
