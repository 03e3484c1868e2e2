"""Initial conditions (host side).

Same classes as ``pararealml/initial_condition.py:18-405``.  Every
vertex-oriented discrete initial state has the static Dirichlet constraints
re-applied (``initial_condition.py:85-89,188-195``), which the GPU solvers rely
on: they take ``discrete_y_0(True)`` as their first state unchanged.
"""

from __future__ import annotations

from abc import ABC, abstractmethod
from copy import deepcopy
from typing import Callable, Optional, Sequence, Tuple

import numpy as np

from .constrained_problem import ConstrainedProblem
from .constraint import apply_constraints_along_last_axis

VectorizedInitialConditionFunction = Callable[[Optional[np.ndarray]], np.ndarray]


class InitialCondition(ABC):
    @abstractmethod
    def y_0(self, x: Optional[np.ndarray]) -> np.ndarray:
        """y at the points ``x`` (``(n, x_dim)``) or the ODE initial vector."""

    @abstractmethod
    def discrete_y_0(self, vertex_oriented: Optional[bool] = None) -> np.ndarray:
        """y at the vertices or cell centres of the mesh."""


class DiscreteInitialCondition(InitialCondition):
    def __init__(
        self,
        cp: ConstrainedProblem,
        y_0: np.ndarray,
        vertex_oriented: Optional[bool] = None,
        interpolation_method: str = "linear",
    ):
        if cp.differential_equation.x_dimension and vertex_oriented is None:
            raise ValueError("vertex orientation must be defined for PDEs")
        if y_0.shape != cp.y_shape(vertex_oriented):
            raise ValueError(
                f"discrete initial value shape {y_0.shape} must match "
                f"constrained problem solution shape {cp.y_shape(vertex_oriented)}"
            )
        self._cp = cp
        self._y_0 = np.array(y_0, dtype=float, copy=True)
        self._vertex_oriented = vertex_oriented
        self._interpolation_method = interpolation_method
        if vertex_oriented:
            apply_constraints_along_last_axis(cp.static_y_vertex_constraints, self._y_0)

    def y_0(self, x: Optional[np.ndarray]) -> np.ndarray:
        if not self._cp.differential_equation.x_dimension:
            return np.copy(self._y_0)
        from scipy.interpolate import interpn

        return interpn(
            self._cp.mesh.axis_coordinates(self._vertex_oriented),
            self._y_0,
            x,
            method=self._interpolation_method,
            bounds_error=False,
            fill_value=None,
        )

    def discrete_y_0(self, vertex_oriented: Optional[bool] = None) -> np.ndarray:
        if vertex_oriented is None:
            vertex_oriented = self._vertex_oriented
        if (
            not self._cp.differential_equation.x_dimension
            or vertex_oriented == self._vertex_oriented
        ):
            return np.copy(self._y_0)
        y_0 = self.y_0(self._cp.mesh.all_index_coordinates(vertex_oriented))
        if vertex_oriented:
            apply_constraints_along_last_axis(self._cp.static_y_vertex_constraints, y_0)
        return y_0


class ConstantInitialCondition(DiscreteInitialCondition):
    def __init__(self, cp: ConstrainedProblem, constant_y_0s: Sequence[float]):
        y_dim = cp.differential_equation.y_dimension
        if len(constant_y_0s) != y_dim:
            raise ValueError(
                f"length of constant y0 values ({len(constant_y_0s)}) must "
                f"match number of y components ({y_dim})"
            )
        ic = np.empty(cp.y_shape(True))
        for i, v in enumerate(constant_y_0s):
            ic[..., i] = v
        super().__init__(cp, ic, True)


class ContinuousInitialCondition(InitialCondition):
    def __init__(
        self,
        cp: ConstrainedProblem,
        y_0_func: VectorizedInitialConditionFunction,
        multipliers: Optional[Sequence[float]] = None,
    ):
        diff_eq = cp.differential_equation
        if multipliers is not None:
            if len(multipliers) != diff_eq.y_dimension:
                raise ValueError(
                    f"length of multipliers ({len(multipliers)}) must match "
                    f"number of y dimensions ({diff_eq.y_dimension})"
                )
            self._multipliers = np.array(multipliers)
        else:
            self._multipliers = np.ones(diff_eq.y_dimension)
        self._cp = cp
        self._y_0_func = y_0_func
        self._discrete_vertices = self._discretize(True)
        self._discrete_cells = self._discretize(False)

    def y_0(self, x: Optional[np.ndarray]) -> np.ndarray:
        return np.multiply(self._y_0_func(x), self._multipliers)

    def discrete_y_0(self, vertex_oriented: Optional[bool] = None) -> np.ndarray:
        return np.copy(self._discrete_vertices if vertex_oriented else self._discrete_cells)

    def _discretize(self, vertex_oriented: bool) -> np.ndarray:
        diff_eq = self._cp.differential_equation
        if not diff_eq.x_dimension:
            y_0 = np.array(self.y_0(None))
            if y_0.shape != self._cp.y_shape():
                raise ValueError(
                    "expected initial condition function output shape to be "
                    f"{self._cp.y_shape()} but got {y_0.shape}"
                )
            return y_0
        x = self._cp.mesh.all_index_coordinates(vertex_oriented, flatten=True)
        y_0 = self.y_0(x)
        if y_0.shape != (len(x), diff_eq.y_dimension):
            raise ValueError(
                "expected initial condition function output shape to be "
                f"{(len(x), diff_eq.y_dimension)} but got {y_0.shape}"
            )
        y_0 = y_0.reshape(self._cp.y_shape(vertex_oriented))
        if vertex_oriented:
            apply_constraints_along_last_axis(self._cp.static_y_vertex_constraints, y_0)
        return y_0


class GaussianInitialCondition(ContinuousInitialCondition):
    """Each component is a (scaled) multivariate normal PDF over the mesh."""

    def __init__(
        self,
        cp: ConstrainedProblem,
        means_and_covs: Sequence[Tuple[np.ndarray, np.ndarray]],
        multipliers: Optional[Sequence[float]] = None,
    ):
        diff_eq = cp.differential_equation
        if not diff_eq.x_dimension:
            raise ValueError("constrained problem must be a PDE")
        if len(means_and_covs) != diff_eq.y_dimension:
            raise ValueError(
                f"number of means and covariances ({len(means_and_covs)}) "
                f"must match number of y dimensions ({diff_eq.y_dimension})"
            )
        for mean, cov in means_and_covs:
            if mean.shape != (diff_eq.x_dimension,):
                raise ValueError(
                    f"expected mean shape to be {(diff_eq.x_dimension,)} but got {mean.shape}"
                )
            if cov.shape != (diff_eq.x_dimension, diff_eq.x_dimension):
                raise ValueError(
                    "expected covariance shape to be "
                    f"{(diff_eq.x_dimension, diff_eq.x_dimension)} but got {cov.shape}"
                )
        self._means_and_covs = deepcopy(means_and_covs)
        super().__init__(cp, self._gaussian, multipliers)

    def _gaussian(self, x: Optional[np.ndarray]) -> np.ndarray:
        """The densities at the Cartesian images of the vertex coordinates
        (reference ``initial_condition.py:232-243, 292-307``)."""
        from scipy.stats import multivariate_normal

        cartesian_x = np.stack(
            to_cartesian_coordinates([x[:, i] for i in range(x.shape[1])], self._cp.mesh.coordinate_system_type),
            axis=-1,
        )
        out = np.empty((len(x), self._cp.differential_equation.y_dimension))
        for i, (mean, cov) in enumerate(self._means_and_covs):
            out[:, i] = multivariate_normal.pdf(cartesian_x, mean=mean, cov=cov)
        return out


def to_cartesian_coordinates(x, from_coordinate_system_type):
    """Curvilinear -> Cartesian coordinates (reference ``mesh.py:561-591``):
    polar (r, theta), cylindrical (r, theta, z), spherical (r, theta, phi)
    with phi measured from the z axis."""
    name = getattr(from_coordinate_system_type, "name", str(from_coordinate_system_type))
    if name == "CARTESIAN":
        return x
    if name == "POLAR":
        return [x[0] * np.cos(x[1]), x[0] * np.sin(x[1])]
    if name == "CYLINDRICAL":
        return [x[0] * np.cos(x[1]), x[0] * np.sin(x[1]), x[2]]
    if name == "SPHERICAL":
        return [x[0] * np.sin(x[2]) * np.cos(x[1]), x[0] * np.sin(x[2]) * np.sin(x[1]), x[0] * np.cos(x[2])]
    raise ValueError(f"unsupported coordinate system type {from_coordinate_system_type}")


def vectorize_ic_function(
    ic_function: Callable[[Optional[Sequence[float]]], Sequence[float]]
) -> VectorizedInitialConditionFunction:
    def vectorized(x: Optional[np.ndarray]) -> np.ndarray:
        if x is None:
            return np.array(ic_function(None))
        return np.array([ic_function(x[i]) for i in range(len(x))])

    return vectorized


_LOG_2PI = float(np.log(2.0 * np.pi))


def _gaussian_terms(cov: np.ndarray):
    """(U, rank log(2 pi) + log pdet) of a covariance matrix, computed the way
    scipy's multivariate normal does (eigendecomposition, pseudo-inverse
    square root of the eigenvalues above its cutoff)."""
    from scipy.linalg import eigh

    s, u = eigh(np.asarray(cov, dtype=np.float64), lower=True)
    eps = 1e6 * np.finfo(s.dtype).eps * np.max(abs(s))
    if np.min(s) < -eps:
        raise ValueError("the input matrix must be positive semidefinite")
    d = s[s > eps]
    s_pinv = np.array([0.0 if abs(x) <= eps else 1.0 / x for x in s], dtype=float)
    return np.multiply(u, np.sqrt(s_pinv)), len(d) * _LOG_2PI + np.sum(np.log(d))


def gaussian_initial_states(cp: ConstrainedProblem, means_and_covs: Sequence, multipliers=None, device=None):
    """Vertex-oriented Gaussian initial states of a batch of instances on
    the GPU, without a host pass per instance.

    ``means_and_covs[b]`` and ``multipliers[b]`` (optional) are what
    ``GaussianInitialCondition(cp, means_and_covs[b], multipliers[b])``
    takes; the result, a CUDA float64 tensor (batch, *vertices, C), holds for
    every b what that object's ``discrete_y_0(True)`` returns (reference
    ``initial_condition.py:150-307``: the densities at the Cartesian images of
    the vertices, times the multipliers, then the static Dirichlet vertex
    constraints) up to the rounding of the device's ``exp``."""
    import torch

    from . import _native

    diff_eq = cp.differential_equation
    dim, comps = diff_eq.x_dimension, diff_eq.y_dimension
    if not dim:
        raise ValueError("constrained problem must be a PDE")
    batch = len(means_and_covs)
    if batch < 1:
        raise ValueError("at least one instance is needed")
    if multipliers is None:
        multipliers = [np.ones(comps)] * batch
    if len(multipliers) != batch:
        raise ValueError("one multiplier sequence per instance is needed")
    n_p = dim + dim * dim + 2
    prm = np.empty((batch, comps, n_p))
    for b, (mcs, mult) in enumerate(zip(means_and_covs, multipliers)):
        if len(mcs) != comps:
            raise ValueError(f"number of means and covariances ({len(mcs)}) must match number of y dimensions "
                             f"({comps})")
        if len(mult) != comps:
            raise ValueError(f"length of multipliers ({len(mult)}) must match number of y dimensions ({comps})")
        for c, (mean, cov) in enumerate(mcs):
            mean = np.asarray(mean, dtype=np.float64)
            cov = np.asarray(cov, dtype=np.float64)
            if mean.shape != (dim,) or cov.shape != (dim, dim):
                raise ValueError(f"expected mean shape {(dim,)} and covariance shape {(dim, dim)}")
            u, c0 = _gaussian_terms(cov)
            prm[b, c, :dim] = mean
            prm[b, c, dim:dim + dim * dim] = u.reshape(-1)
            prm[b, c, -2] = c0
            prm[b, c, -1] = float(mult[c])
    mesh = cp.mesh
    x = mesh.all_index_coordinates(True, flatten=True)
    cart = np.ascontiguousarray(np.stack(
        to_cartesian_coordinates([x[:, i] for i in range(dim)], mesh.coordinate_system_type), axis=-1),
        dtype=np.float64)
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    xd = torch.from_numpy(cart).to(dev)
    pd = torch.from_numpy(prm).to(dev)
    out = torch.empty((batch,) + tuple(mesh.vertices_shape) + (comps,), dtype=torch.float64, device=dev)
    _native.check(_native.lib().prml_gaussian_states(xd.data_ptr(), len(cart), dim, pd.data_ptr(), batch, comps,
                                                     out.data_ptr(), torch.cuda.current_stream(dev).cuda_stream),
                  "Gaussian initial states")
    cons = cp.static_y_vertex_constraints
    if cons is not None:
        dense = np.full(tuple(mesh.vertices_shape) + (comps,), np.nan)
        apply_constraints_along_last_axis(cons, dense)
        if np.any(~np.isnan(dense)):
            dd = torch.from_numpy(dense).to(dev)
            out = torch.where(torch.isnan(dd), out, dd.expand_as(out))
    return out
