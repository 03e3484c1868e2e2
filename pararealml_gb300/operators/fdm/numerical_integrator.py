"""Explicit integrators of the GPU FDM path.

Same classes as ``pararealml/operators/fdm/numerical_integrator.py:42-132``.
On the GPU an integrator is a kind (number of stages) that selects the
stage schedule of the fused step kernel; the arithmetic of each stage
(``y + d_t * f``, ``y + k1 / 2`` ..., ``(k1 + 2k2 + 2k3 + k4) / 6``) is the
reference's and lives in ``csrc/fdm_step.cuh``.  The implicit methods of the
reference (backward Euler, Crank-Nicolson: scipy secant iterations,
``numerical_integrator.py:135-270``) have no GPU kernel and are rejected.
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


_BY_NAME = {
    "ForwardEulerMethod": codegen.FORWARD_EULER,
    "ExplicitMidpointMethod": codegen.EXPLICIT_MIDPOINT,
    "RK4": codegen.RK4,
}


def integrator_kind(integrator) -> int:
    """Stage count of an integrator object (this package's or the reference's)."""
    kind = getattr(integrator, "kind", None)
    if isinstance(kind, int) and kind in _BY_NAME.values():
        return kind
    name = type(integrator).__name__
    if name in _BY_NAME:
        return _BY_NAME[name]
    raise NotImplementedError(
        f"{name} has no GPU kernel: the GPU FDM path supports ForwardEulerMethod, "
        "ExplicitMidpointMethod and RK4"
    )
