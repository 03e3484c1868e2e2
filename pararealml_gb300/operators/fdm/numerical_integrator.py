"""Integrators of the GPU FDM path.

Same classes and constructors as ``pararealml/operators/fdm/
numerical_integrator.py:42-270``.  An explicit integrator is a kind (number
of stages) that selects the stage schedule of the fused step kernel; the
arithmetic of each stage (``y + d_t * f``, ``y + k1 / 2`` ...,
``(k1 + 2k2 + 2k3 + k4) / 6``) is the reference's and lives in
``csrc/fdm_step.cuh``.  The implicit methods (backward Euler,
Crank-Nicolson) solve each step with the reference's element-wise secant
iteration: the generated right-hand-side kernel plus ``csrc/prml_implicit.cu``,
driven by ``engine.StencilPlan``.
"""

from __future__ import annotations

from ... import codegen


class NumericalIntegrator:
    kind: int = 0


class ForwardEulerMethod(NumericalIntegrator):
    kind = codegen.FORWARD_EULER


class ExplicitMidpointMethod(NumericalIntegrator):
    kind = codegen.EXPLICIT_MIDPOINT


class RK4(NumericalIntegrator):
    kind = codegen.RK4


class ImplicitMethod(NumericalIntegrator):
    """numerical_integrator.py:135-155: secant tolerance and iteration cap."""

    def __init__(self, tol: float = 1.48e-8, max_iterations: int = 50):
        if tol < 0.0:
            raise ValueError("tolerance must be non-negative")
        if max_iterations <= 0:
            raise ValueError("number of maximum iterations must be greater than 0")
        self._tol = tol
        self._max_iterations = max_iterations


class BackwardEulerMethod(ImplicitMethod):
    kind = codegen.BACKWARD_EULER


class CrankNicolsonMethod(ImplicitMethod):
    """numerical_integrator.py:224-248: ``a`` weighs the backward Euler term."""

    kind = codegen.CRANK_NICOLSON

    def __init__(self, a: float = 0.5, tol: float = 1.48e-8, max_iterations: int = 50):
        if not (0.0 <= a <= 1.0):
            raise ValueError("the value of 'a' must be between 0 and 1")
        self._a = a
        self._b = 1.0 - a
        super().__init__(tol, max_iterations)


_BY_NAME = {
    "ForwardEulerMethod": codegen.FORWARD_EULER,
    "ExplicitMidpointMethod": codegen.EXPLICIT_MIDPOINT,
    "RK4": codegen.RK4,
    "BackwardEulerMethod": codegen.BACKWARD_EULER,
    "CrankNicolsonMethod": codegen.CRANK_NICOLSON,
}


def integrator_kind(integrator) -> int:
    """Kind of an integrator object (this package's or the reference's)."""
    kind = getattr(integrator, "kind", None)
    if isinstance(kind, int) and kind in _BY_NAME.values():
        return kind
    name = type(integrator).__name__
    if name in _BY_NAME:
        return _BY_NAME[name]
    raise NotImplementedError(
        f"{name} has no GPU kernel: the GPU FDM path supports ForwardEulerMethod, "
        "ExplicitMidpointMethod, RK4, BackwardEulerMethod and CrankNicolsonMethod"
    )


def implicit_settings(integrator) -> dict:
    """Secant settings of an implicit integrator (this package's or the
    reference's: the same private attributes)."""
    kind = integrator_kind(integrator)
    if kind not in codegen.IMPLICIT:
        raise ValueError("not an implicit integrator")
    return {
        "a": float(getattr(integrator, "_a", 1.0)) if kind == codegen.CRANK_NICOLSON else 1.0,
        "tol": float(integrator._tol),
        "max_iterations": int(integrator._max_iterations),
        "crank_nicolson": kind == codegen.CRANK_NICOLSON,
    }
