from .fdm_operator import FDMOperator
from .numerical_differentiator import NumericalDifferentiator, ThreePointCentralDifferenceMethod
from .numerical_integrator import (
    ExplicitMidpointMethod,
    ForwardEulerMethod,
    NumericalIntegrator,
    RK4,
)

__all__ = [
    "FDMOperator",
    "NumericalDifferentiator",
    "ThreePointCentralDifferenceMethod",
    "NumericalIntegrator",
    "ForwardEulerMethod",
    "ExplicitMidpointMethod",
    "RK4",
]
