from .parareal_operator import FDMCoarsePropagator, PararealOperator

__all__ = ["PararealOperator", "FDMCoarsePropagator"]
