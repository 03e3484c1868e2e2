from .fdm_operator import FDMOperator
from .numerical_differentiator import NumericalDifferentiator, ThreePointCentralDifferenceMethod
from .numerical_integrator import (
    BackwardEulerMethod,
    CrankNicolsonMethod,
    ExplicitMidpointMethod,
    ForwardEulerMethod,
    ImplicitMethod,
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
    "ImplicitMethod",
    "BackwardEulerMethod",
    "CrankNicolsonMethod",
]
