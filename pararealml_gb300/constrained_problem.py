"""A differential equation constrained by a mesh and boundary conditions.

Same surface as ``pararealml/constrained_problem.py:15-476``.  Boundary
condition functions are evaluated on the boundary points of each axis into
``(x_dim, y_dim)`` object arrays of ``(lower, upper)`` ``Constraint`` pairs, one
for y and one for the normal derivative of y (``:303-476``), and the y
constraints are folded into one whole-field ``Constraint`` per component in
which later axes overwrite earlier ones at corners (``:262-301``).  The GPU
lowering reads these tables and turns them into dense NaN-masked face arrays.
"""

from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np

from .boundary_condition import BoundaryCondition
from .constraint import Constraint
from .differential_equation import DifferentialEquation
from .mesh import Mesh

BoundaryConditionPair = Tuple[BoundaryCondition, BoundaryCondition]


class ConstrainedProblem:
    def __init__(
        self,
        diff_eq: DifferentialEquation,
        mesh: Optional[Mesh] = None,
        boundary_conditions: Optional[Sequence[BoundaryConditionPair]] = None,
    ):
        self._diff_eq = diff_eq
        if diff_eq.x_dimension:
            if mesh is None:
                raise ValueError("mesh cannot be None for PDEs")
            if mesh.dimensions != diff_eq.x_dimension:
                raise ValueError(
                    f"mesh dimensions ({mesh.dimensions}) must match "
                    "differential equation spatial dimensions "
                    f"({diff_eq.x_dimension})"
                )
            if boundary_conditions is None:
                raise ValueError("boundary conditions cannot be None for PDEs")
            if len(boundary_conditions) != diff_eq.x_dimension:
                raise ValueError(
                    "number of boundary condition pairs "
                    f"({len(boundary_conditions)}) must match differential "
                    f"equation spatial dimensions ({diff_eq.x_dimension})"
                )
            self._mesh = mesh
            self._boundary_conditions = tuple(boundary_conditions)
            self._y_vertices_shape = mesh.vertices_shape + (diff_eq.y_dimension,)
            self._y_cells_shape = mesh.cells_shape + (diff_eq.y_dimension,)
            self._are_all_bcs_static = np.bool_(
                all(lo.is_static and hi.is_static for lo, hi in boundary_conditions)
            )
            self._are_there_bcs_on_y = np.bool_(
                any(lo.has_y_condition or hi.has_y_condition for lo, hi in boundary_conditions)
            )
            self._boundary_vertex_constraints = None
            self._boundary_cell_constraints = None
            self._boundary_vertex_constraints = self.create_boundary_constraints(True)
            self._boundary_cell_constraints = self.create_boundary_constraints(False)
            for pair in (self._boundary_vertex_constraints, self._boundary_cell_constraints):
                pair[0].setflags(write=False)
                pair[1].setflags(write=False)
            self._y_vertex_constraints = self.create_y_vertex_constraints(
                self._boundary_vertex_constraints[0]
            )
            self._y_vertex_constraints.setflags(write=False)
        else:
            self._mesh = None
            self._boundary_conditions = None
            self._y_vertices_shape = self._y_cells_shape = (diff_eq.y_dimension,)
            self._are_all_bcs_static = np.bool_(False)
            self._are_there_bcs_on_y = np.bool_(False)
            self._boundary_vertex_constraints = None
            self._boundary_cell_constraints = None
            self._y_vertex_constraints = None

    differential_equation = property(lambda self: self._diff_eq)
    mesh = property(lambda self: self._mesh)
    boundary_conditions = property(lambda self: self._boundary_conditions)
    y_vertices_shape = property(lambda self: self._y_vertices_shape)
    y_cells_shape = property(lambda self: self._y_cells_shape)
    are_all_boundary_conditions_static = property(lambda self: self._are_all_bcs_static)
    are_there_boundary_conditions_on_y = property(lambda self: self._are_there_bcs_on_y)
    static_boundary_vertex_constraints = property(
        lambda self: self._boundary_vertex_constraints
    )
    static_boundary_cell_constraints = property(lambda self: self._boundary_cell_constraints)
    static_y_vertex_constraints = property(lambda self: self._y_vertex_constraints)

    def y_shape(self, vertex_oriented: Optional[bool] = None) -> Tuple[int, ...]:
        return self._y_vertices_shape if vertex_oriented else self._y_cells_shape

    def static_boundary_constraints(self, vertex_oriented: bool):
        return (
            self._boundary_vertex_constraints
            if vertex_oriented
            else self._boundary_cell_constraints
        )

    def create_y_vertex_constraints(
        self, y_boundary_vertex_constraints: Optional[np.ndarray]
    ) -> Optional[np.ndarray]:
        """One whole-field ``Constraint`` per y component; later axes win at corners."""
        diff_eq = self._diff_eq
        if not diff_eq.x_dimension or y_boundary_vertex_constraints is None:
            return None
        ndim = len(self._y_vertices_shape)
        out = np.empty(diff_eq.y_dimension, dtype=object)
        field = np.empty(self._y_vertices_shape[:-1] + (1,))
        for y_ind in range(diff_eq.y_dimension):
            field.fill(np.nan)
            for axis in range(diff_eq.x_dimension):
                for side, c in enumerate(y_boundary_vertex_constraints[axis, y_ind]):
                    if c is None:
                        continue
                    sl = [slice(None)] * ndim
                    sl[axis] = slice(-1, None) if side else slice(0, 1)
                    c.apply(field[tuple(sl)])
            mask = ~np.isnan(field)
            out[y_ind] = Constraint(field[mask], mask)
        return out

    def create_boundary_constraints(
        self, vertex_oriented: bool, t: Optional[float] = None
    ) -> Tuple[Optional[np.ndarray], Optional[np.ndarray]]:
        """``(y, dy/dn)`` tables of ``(lower, upper)`` constraint pairs per axis/component."""
        diff_eq = self._diff_eq
        if not diff_eq.x_dimension:
            return None, None
        coords = self._mesh.all_index_coordinates(vertex_oriented)
        y_pairs = np.empty((diff_eq.x_dimension, diff_eq.y_dimension), dtype=object)
        d_y_pairs = np.empty((diff_eq.x_dimension, diff_eq.y_dimension), dtype=object)
        for axis, bc_pair in enumerate(self._boundary_conditions):
            y_row, d_y_row = self._axis_pairs(bc_pair, coords, axis, vertex_oriented, t)
            y_pairs[axis, :] = y_row
            d_y_pairs[axis, :] = d_y_row
        return y_pairs, d_y_pairs

    def _axis_pairs(self, bc_pair, coords, axis, vertex_oriented, t):
        y_dim = self._diff_eq.y_dimension
        static = self.static_boundary_constraints(vertex_oriented)
        per_side_y: List[Sequence[Optional[Constraint]]] = []
        per_side_dy: List[Sequence[Optional[Constraint]]] = []
        for side, bc in enumerate(bc_pair):
            if not bc.is_static and t is None:
                per_side_y.append([None] * y_dim)
                per_side_dy.append([None] * y_dim)
            elif bc.is_static and static is not None:
                per_side_y.append([static[0][axis, i][side] for i in range(y_dim)])
                per_side_dy.append([static[1][axis, i][side] for i in range(y_dim)])
            else:
                sl = [slice(None)] * coords.ndim
                sl[axis] = slice(-1, None) if side else slice(0, 1)
                face = np.copy(coords[tuple(sl)])
                face[..., axis] = self._mesh.vertex_axis_coordinates[axis][-side]
                per_side_y.append(
                    self._face_constraints(bc.has_y_condition, bc.y_condition, face, t)
                )
                per_side_dy.append(
                    self._face_constraints(bc.has_d_y_condition, bc.d_y_condition, face, t)
                )
        y_row = np.empty(y_dim, dtype=object)
        y_row[:] = list(zip(*per_side_y))
        d_y_row = np.empty(y_dim, dtype=object)
        d_y_row[:] = list(zip(*per_side_dy))
        return y_row, d_y_row

    def _face_constraints(self, has_condition, fn, face, t):
        x_dim = self._diff_eq.x_dimension
        y_dim = self._diff_eq.y_dimension
        if not has_condition:
            return [None] * y_dim
        x = face.reshape((-1, x_dim))
        values = fn(x, t)
        if values.shape != (len(x), y_dim):
            raise ValueError(
                "expected boundary condition function output shape to be "
                f"{(len(x), y_dim)} but got {values.shape}"
            )
        values = values.reshape(face.shape[:-1] + (y_dim,))
        out = []
        for i in range(y_dim):
            v = values[..., i: i + 1]
            mask = ~np.isnan(v)
            out.append(Constraint(v[mask], mask))
        return out
