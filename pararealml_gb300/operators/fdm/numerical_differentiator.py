"""Finite difference schemes of the GPU FDM path.

``ThreePointCentralDifferenceMethod`` mirrors the reference class
(``pararealml/operators/fdm/numerical_differentiator.py:999-1242``); its
stencils (zero-halo first derivatives with Neumann overwrite, Neumann ghost
vertices for second derivatives) are implemented by the fused kernel in
``csrc/fdm_step.cuh``.  ``tol`` is the Jacobi tolerance of the
anti-Laplacian, kept for interface parity.
"""

from __future__ import annotations


class NumericalDifferentiator:
    def __init__(self, tol: float = 1e-3):
        if tol < 0.0:
            raise ValueError("tolerance must be non-negative")
        self._tol = tol


class ThreePointCentralDifferenceMethod(NumericalDifferentiator):
    pass


def check_differentiator(differentiator) -> None:
    if type(differentiator).__name__ != "ThreePointCentralDifferenceMethod":
        raise NotImplementedError(
            "the GPU FDM path implements the ThreePointCentralDifferenceMethod stencils only"
        )
