"""Solutions of initial value problems.

Same surface as ``pararealml/solution.py:25-258`` (``t_coordinates``,
``discrete_y``, ``y``, ``diff``, ``d_t``, ``vertex_oriented``), with one
GB300-side addition: the trajectory may be held as a CUDA tensor
(``device_y``) and is only copied to host memory when a host array is asked
for, so that a caller who needs the final state or a strided trajectory does
not pay for a full host copy.  ``discrete_y`` always returns a host numpy
array of shape ``(len(t), *y_shape)`` exactly as the reference does.
"""

from __future__ import annotations

import os
import threading
from concurrent.futures import ThreadPoolExecutor
from typing import List, NamedTuple, Optional, Sequence

import numpy as np

from .constraint import apply_constraints_along_last_axis
from .initial_value_problem import InitialValueProblem

# arrays from this size on are copied by several host threads (numpy
# releases the GIL while it copies; one thread moves ~16 GB/s)
_PARALLEL_COPY_BYTES = 16 << 20
_copy_pool: Optional[ThreadPoolExecutor] = None
_copy_lock = threading.Lock()


def _copy(a: np.ndarray) -> np.ndarray:
    """``np.copy(a)``, split into contiguous chunks over a few threads
    for large C-contiguous arrays."""
    global _copy_pool
    threads = min(8, os.cpu_count() or 1)
    if a.nbytes < _PARALLEL_COPY_BYTES or threads < 2 or not a.flags.c_contiguous:
        return np.copy(a)
    with _copy_lock:
        if _copy_pool is None:
            _copy_pool = ThreadPoolExecutor(max_workers=threads, thread_name_prefix="prml-copy")
    out = np.empty_like(a)
    src, dst = a.reshape(-1), out.reshape(-1)
    bounds = np.linspace(0, src.size, threads + 1).astype(np.int64)
    list(_copy_pool.map(lambda k: np.copyto(dst[bounds[k]:bounds[k + 1]], src[bounds[k]:bounds[k + 1]]),
                        range(threads)))
    return out


class Diffs(NamedTuple):
    matching_time_points: np.ndarray
    differences: Sequence[np.ndarray]


class Solution:
    def __init__(
        self,
        ivp: InitialValueProblem,
        t_coordinates: np.ndarray,
        discrete_y,
        vertex_oriented: Optional[bool] = None,
        d_t: Optional[float] = None,
        copy: bool = True,
    ):
        """``copy=False`` (not in the reference, which always copies,
        ``solution.py:71-72``) keeps a caller-owned host array as is."""
        if t_coordinates.ndim != 1:
            raise ValueError(
                f"number of t coordinate dimensions ({t_coordinates.ndim}) must be 1"
            )
        if len(t_coordinates) == 0:
            raise ValueError("length of t coordinates must be greater than 0")
        cp = ivp.constrained_problem
        if cp.differential_equation.x_dimension and vertex_oriented is None:
            raise ValueError("vertex orientation must be defined for solutions to PDEs")
        y_shape = cp.y_shape(vertex_oriented)
        if tuple(discrete_y.shape) != (len(t_coordinates),) + tuple(y_shape):
            raise ValueError(
                "expected solution shape to be "
                f"{((len(t_coordinates),) + tuple(y_shape))} but got {tuple(discrete_y.shape)}"
            )
        self._ivp = ivp
        self._t_coordinates = np.array(t_coordinates, copy=True)
        self._t_coordinates.setflags(write=False)
        self._vertex_oriented = vertex_oriented
        if isinstance(discrete_y, np.ndarray):
            self._host_y = _copy(discrete_y) if copy else discrete_y
            self._device_y = None
        else:  # a torch tensor (on a CUDA device) owned by this solution
            self._host_y = None
            self._device_y = discrete_y
        if d_t is None:
            d_t = 0.0 if len(t_coordinates) == 1 else t_coordinates[1] - t_coordinates[0]
        self._d_t = d_t

    initial_value_problem = property(lambda self: self._ivp)
    vertex_oriented = property(lambda self: self._vertex_oriented)
    d_t = property(lambda self: self._d_t)
    t_coordinates = property(lambda self: self._t_coordinates)

    @property
    def device_y(self):
        """The trajectory as a CUDA tensor if the solver kept it on the device."""
        return self._device_y

    def _host(self) -> np.ndarray:
        if self._host_y is None:
            self._host_y = self._device_y.detach().to("cpu").numpy().astype(np.float64, copy=False)
        return self._host_y

    def y(self, x: Optional[np.ndarray] = None, interpolation_method: str = "linear") -> np.ndarray:
        cp = self._ivp.constrained_problem
        diff_eq = cp.differential_equation
        if not diff_eq.x_dimension:
            return _copy(self._host())
        from scipy.interpolate import interpn

        y = interpn(
            cp.mesh.axis_coordinates(self._vertex_oriented),
            np.moveaxis(self._host(), 0, -2),
            x,
            method=interpolation_method,
            bounds_error=False,
            fill_value=None,
        )
        y = np.moveaxis(y, -2, 0)
        y = y.reshape((len(self._t_coordinates),) + x.shape[:-1] + (diff_eq.y_dimension,))
        return np.ascontiguousarray(y)

    def discrete_y(
        self, vertex_oriented: Optional[bool] = None, interpolation_method: str = "linear"
    ) -> np.ndarray:
        if vertex_oriented is None:
            vertex_oriented = self._vertex_oriented
        cp = self._ivp.constrained_problem
        if not cp.differential_equation.x_dimension or self._vertex_oriented == vertex_oriented:
            return _copy(self._host())
        x = cp.mesh.all_index_coordinates(vertex_oriented)
        out = self.y(x, interpolation_method)
        if vertex_oriented:
            apply_constraints_along_last_axis(cp.static_y_vertex_constraints, out)
        return out

    def diff(self, solutions: Sequence["Solution"], atol: float = 1e-8) -> Diffs:
        """Differences to other solutions at the time points all of them share."""
        if len(solutions) == 0:
            raise ValueError("length of solutions must be greater than 0")
        times = [self._t_coordinates] + [s.t_coordinates for s in solutions]
        steps = [self._d_t] + [s.d_t for s in solutions]
        others = [s.discrete_y(self._vertex_oriented) for s in solutions]
        own = self._host()
        base = int(np.argmin([len(tp) for tp in times]))
        matches: List[float] = []
        diffs: List[List[np.ndarray]] = [[] for _ in solutions]
        for i, t in enumerate(times[base]):
            idx = []
            for j, tp in enumerate(times):
                if j == base:
                    idx.append(i)
                    continue
                k = int(round((t - tp[0]) / steps[j]))
                if 0 <= k < len(tp) and np.isclose(t, tp[k], atol=atol, rtol=0.0):
                    idx.append(k)
                else:
                    break
            else:
                matches.append(t)
                for j, other in enumerate(others):
                    diffs[j].append(other[idx[j + 1]] - own[idx[0]])
        return Diffs(np.array(matches), [np.array(d) for d in diffs])
