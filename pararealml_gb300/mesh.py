"""Uniform hyper-rectangular meshes (host side).

Mirrors ``pararealml/mesh.py:20-488``: a ``Mesh`` is defined by per-axis
intervals and step sizes; vertex counts are ``round(L/dx + 1)`` per axis
(``mesh.py:305-325``) and axis coordinates are ``linspace`` grids
(``mesh.py:327-356``).  The GPU path supports Cartesian meshes; the
coordinate-system enum is kept so that curvilinear problems are rejected with
a clear error rather than silently mis-solved.
"""

from __future__ import annotations

from enum import Enum
from typing import Sequence, Tuple

import numpy as np

SpatialDomainInterval = Tuple[float, float]


class CoordinateSystem(Enum):
    CARTESIAN = 0
    POLAR = 1
    CYLINDRICAL = 2
    SPHERICAL = 3


class Mesh:
    """A uniform grid over a hyper-rectangular spatial domain."""

    def __init__(
        self,
        x_intervals: Sequence[SpatialDomainInterval],
        d_x: Sequence[float],
        coordinate_system_type: CoordinateSystem = CoordinateSystem.CARTESIAN,
    ):
        if len(x_intervals) == 0:
            raise ValueError("number of spatial domain intervals must be greater than 0")
        if len(x_intervals) != len(d_x):
            raise ValueError(
                f"number of spatial domain intervals ({len(x_intervals)}) "
                f"must match number of spatial step sizes ({len(d_x)})"
            )
        if any(hi <= lo for lo, hi in x_intervals):
            raise ValueError(
                "upper bound of every spatial domain interval must be greater "
                "than its lower bound"
            )
        if any(h <= 0.0 for h in d_x):
            raise ValueError("all spatial step sizes must be greater than 0")
        self._x_intervals = tuple(tuple(iv) for iv in x_intervals)
        self._d_x = tuple(d_x)
        self._coordinate_system_type = coordinate_system_type
        self._dimensions = len(x_intervals)
        self._vertices_shape = self._shape(True)
        self._cells_shape = self._shape(False)
        self._vertex_axis_coordinates = self._axis_coords(True)
        self._cell_center_axis_coordinates = self._axis_coords(False)
        self._vertex_coordinate_grids = self._grids(True)
        self._cell_center_coordinate_grids = self._grids(False)

    x_intervals = property(lambda self: self._x_intervals)
    d_x = property(lambda self: self._d_x)
    coordinate_system_type = property(lambda self: self._coordinate_system_type)
    dimensions = property(lambda self: self._dimensions)
    vertices_shape = property(lambda self: self._vertices_shape)
    cells_shape = property(lambda self: self._cells_shape)
    vertex_axis_coordinates = property(lambda self: self._vertex_axis_coordinates)
    cell_center_axis_coordinates = property(
        lambda self: self._cell_center_axis_coordinates
    )
    vertex_coordinate_grids = property(lambda self: self._vertex_coordinate_grids)
    cell_center_coordinate_grids = property(
        lambda self: self._cell_center_coordinate_grids
    )

    def shape(self, vertex_oriented: bool) -> Tuple[int, ...]:
        return self._vertices_shape if vertex_oriented else self._cells_shape

    def axis_coordinates(self, vertex_oriented: bool) -> Tuple[np.ndarray, ...]:
        return (
            self._vertex_axis_coordinates
            if vertex_oriented
            else self._cell_center_axis_coordinates
        )

    def coordinate_grids(self, vertex_oriented: bool) -> Tuple[np.ndarray, ...]:
        return (
            self._vertex_coordinate_grids
            if vertex_oriented
            else self._cell_center_coordinate_grids
        )

    def all_index_coordinates(
        self, vertex_oriented: bool, flatten: bool = False
    ) -> np.ndarray:
        coords = np.stack(self.coordinate_grids(vertex_oriented), axis=-1)
        return coords.reshape((-1, self._dimensions)) if flatten else coords

    def _shape(self, vertex_oriented: bool) -> Tuple[int, ...]:
        return tuple(
            round((hi - lo) / h + vertex_oriented)
            for (lo, hi), h in zip(self._x_intervals, self._d_x)
        )

    def _axis_coords(self, vertex_oriented: bool) -> Tuple[np.ndarray, ...]:
        shape = self._shape(vertex_oriented)
        out = []
        for (lo, hi), h, n in zip(self._x_intervals, self._d_x, shape):
            if not vertex_oriented:
                lo, hi = lo + h / 2.0, hi - h / 2.0
            c = np.linspace(lo, hi, n)
            c.setflags(write=False)
            out.append(c)
        return tuple(out)

    def _grids(self, vertex_oriented: bool) -> Tuple[np.ndarray, ...]:
        grids = np.meshgrid(*self._axis_coords(vertex_oriented), indexing="ij")
        for g in grids:
            g.setflags(write=False)
        return tuple(grids)
