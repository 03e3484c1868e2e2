"""CPU oracle: numpy restatement of PararealML's FDM hot path.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke``
and ``bench.py``'s CPU-baseline arm as the checker; the product package never
imports it.

Pinned against the reference (ViktorC/PararealML) by the golden fixtures in
``tests/golden`` (generated by running the reference itself,
``tests/golden/make_golden.py``) and by the reference's own known-answer
stencil and integrator tests, restated in ``tests/test_oracle.py``.

Every function follows the reference's whole-array numpy formulation so that
timing it on the host cores is representative of the reference's own speed:

* ``derivative``        <- numerical_differentiator.py:1012-1057
* ``second_derivative`` <- numerical_differentiator.py:1059-1095, 1188-1242
* ``gradient/hessian/divergence/curl/laplacian`` (Cartesian branches)
                        <- numerical_differentiator.py:114-156, 175-227,
                           310-346, 402-459, 592-634
* ``anti_laplacian``    <- numerical_differentiator.py:872-927 (Jacobi loop),
                           1097-1186 (_next_anti_laplacian_estimate)
* ``FDMStepper``        <- fdm_operator.py:79-165 (y_next_function) with
                           numerical_integrator.py:42-132 (FE, midpoint, RK4)
                           and 135-270 (backward Euler, Crank-Nicolson)
* ``secant_solve``      <- the vectorised secant method of
                           scipy.optimize.newton without a derivative
                           (scipy/optimize/_zeros_py.py, _array_newton),
                           which ImplicitMethod._solve calls
                           (numerical_integrator.py:157-176); pinned against
                           scipy itself in tests/test_oracle.py
* ``fdm_solve``         <- fdm_operator.py:48-77
The problem description is read from a constrained-problem object through
the same public attributes the reference exposes
(``static_boundary_vertex_constraints``, ``static_y_vertex_constraints``,
``mesh``, ``differential_equation``).
"""

from __future__ import annotations

from typing import Callable, List, Optional, Sequence

import numpy as np
import sympy as sp

FE, MIDPOINT, RK4 = "fe", "midpoint", "rk4"
BACKWARD_EULER, CRANK_NICOLSON = "be", "cn"


def secant_solve(func, x0: np.ndarray, tol: float = 1.48e-8, maxiter: int = 50):
    """Element-wise secant iteration on a whole array (the published method
    of scipy.optimize.newton for array x0 and no derivative).

    Returns (root, iterations, warning or None); raises RuntimeError when
    every element fails to converge.  Every element takes the secant step
    x_new = x1 - q1 (x1 - x0) / (q1 - q0) where q1 != q0; elements whose two
    residuals are equal are set once to the midpoint of their last two
    iterates and then left alone; the loop ends when every element that
    stepped moved by less than tol, when no residual changed, or after
    maxiter steps."""
    p = np.array(x0, dtype=np.float64, copy=True)
    failures = np.ones(p.shape, dtype=bool)
    nz = np.ones(p.shape, dtype=bool)
    dx = np.finfo(float).eps ** 0.33
    p1 = p * (1 + dx) + np.where(p >= 0, dx, -dx)
    q0 = np.asarray(func(p))
    q1 = np.asarray(func(p1))
    active = np.ones(p.shape, dtype=bool)
    it = 0
    for it in range(1, maxiter + 1):
        nz = q1 != q0
        if not nz.any():
            p = (p1 + p) / 2.0
            break
        step = (q1 * (p1 - p))[nz] / (q1 - q0)[nz]
        p = np.array(p, dtype=np.float64)
        p[nz] = p1[nz] - step
        mid = ~nz & active
        p[mid] = (p1 + p)[mid] / 2.0
        active &= nz
        failures[nz] = np.abs(step) >= tol
        if not failures[nz].any():
            break
        p1, p = p, p1
        q0 = q1
        q1 = np.asarray(func(p1))
    warning = None
    zero = ~nz & failures
    if zero.any():
        moved = zero & (p1 != p)
        if moved.any():
            warning = f"RMS of {np.sqrt(sum((p1[moved] - p[moved]) ** 2)):g} reached"
    elif failures.any():
        if failures.all():
            raise RuntimeError(f"all failed to converge after {maxiter:d} iterations")
        warning = f"some failed to converge after {maxiter:d} iterations"
    return p, it, warning


# ---------------------------------------------------------------- constraints
def apply_mask(values: np.ndarray, mask: np.ndarray, array: np.ndarray) -> np.ndarray:
    """``Constraint.apply`` (constraint.py:43-58): array[..., mask] = values."""
    array[..., mask] = values
    return array


def apply_y_constraints(constraints, array: np.ndarray) -> np.ndarray:
    """``apply_constraints_along_last_axis`` (constraint.py:104-131)."""
    if constraints is None:
        return array
    for i, c in enumerate(constraints):
        if c is not None:
            apply_mask(c.values, c.mask, array[..., i: i + 1])
    return array


# ---------------------------------------------------------------- stencils
def derivative(y: np.ndarray, d_x: float, axis: int, pairs: Sequence) -> np.ndarray:
    """Zero-halo central difference; Neumann values overwrite boundary rows."""
    if y.shape[axis] <= 2:
        raise ValueError(f"y must contain at least 3 points along x-axis ({axis})")
    halo = np.zeros(y.shape[:axis] + (1,) + y.shape[axis + 1:])
    ext = np.concatenate([halo, y, halo], axis=axis)
    sl = [slice(None)] * y.ndim
    sl[axis] = slice(0, -2)
    prev = ext[tuple(sl)]
    sl[axis] = slice(2, None)
    nxt = ext[tuple(sl)]
    d = (nxt - prev) / (2.0 * d_x)
    sl[axis] = slice(None)
    for comp, pair in enumerate(pairs):
        if pair is None:
            continue
        sl[-1] = slice(comp, comp + 1)
        if pair[0] is not None:
            sl[axis] = slice(0, 1)
            apply_mask(pair[0].values, pair[0].mask, d[tuple(sl)])
        if pair[1] is not None:
            sl[axis] = slice(-1, None)
            apply_mask(pair[1].values, pair[1].mask, d[tuple(sl)])
    return d


def _halos(y: np.ndarray, axis: int, d_x: float, pairs: Sequence) -> np.ndarray:
    sl = [slice(None)] * y.ndim
    sl[axis] = slice(1, 2)
    lo_adj = y[tuple(sl)]
    sl[axis] = slice(-2, -1)
    hi_adj = y[tuple(sl)]
    lo = np.zeros_like(lo_adj)
    hi = np.zeros_like(hi_adj)
    for comp, pair in enumerate(pairs):
        if pair is None:
            continue
        if pair[0] is not None:  # ghost = y[1] - 2 dx g
            m = pair[0].mask
            lo[..., comp: comp + 1][..., m] = lo_adj[..., comp: comp + 1][..., m] + (-2.0 * d_x) * pair[0].values
        if pair[1] is not None:  # ghost = y[n-2] + 2 dx g
            m = pair[1].mask
            hi[..., comp: comp + 1][..., m] = hi_adj[..., comp: comp + 1][..., m] + (2.0 * d_x) * pair[1].values
    return np.concatenate([lo, y, hi], axis=axis)


def second_derivative(y, d_x1, d_x2, a1, a2, pairs) -> np.ndarray:
    if a1 != a2:
        first = derivative(y, d_x1, a1, pairs)
        return derivative(first, d_x2, a2, [None] * y.shape[-1])
    if y.shape[a1] <= 2:
        raise ValueError(f"y must contain at least 3 points along x-axis ({a1})")
    ext = _halos(y, a1, d_x1, pairs)
    sl = [slice(None)] * y.ndim
    sl[a1] = slice(0, -2)
    prev = ext[tuple(sl)]
    sl[a1] = slice(1, -1)
    cur = ext[tuple(sl)]
    sl[a1] = slice(2, None)
    nxt = ext[tuple(sl)]
    return (nxt - 2.0 * cur + prev) / (d_x1 * d_x2)


def _dbc(dbc, n_axes, n_comp):
    if dbc is None:
        out = np.empty((n_axes, n_comp), dtype=object)
        out.fill(None)
        return out
    return dbc


def gradient(y, d_x, axis, dbc=None):
    dbc = _dbc(dbc, len(d_x), y.shape[-1])
    return derivative(y, d_x[axis], axis, dbc[axis])


def hessian(y, d_x, a1, a2, dbc=None):
    dbc = _dbc(dbc, len(d_x), y.shape[-1])
    return second_derivative(y, d_x[a1], d_x[a2], a1, a2, dbc[a1])


def laplacian(y, d_x, dbc=None):
    dbc = _dbc(dbc, len(d_x), y.shape[-1])
    out = np.zeros_like(y)
    for axis in range(y.ndim - 1):
        out += second_derivative(y, d_x[axis], d_x[axis], axis, axis, dbc[axis, :])
    return out


def divergence(y, d_x, dbc=None):
    if y.shape[-1] != y.ndim - 1:
        raise ValueError("number of y components must match number of x dimensions")
    dbc = _dbc(dbc, len(d_x), y.shape[-1])
    out = np.zeros(y.shape[:-1] + (1,))
    for i in range(y.shape[-1]):
        out += derivative(y[..., i: i + 1], d_x[i], i, dbc[i, i: i + 1])
    return out


def curl2d(y, d_x, dbc=None):
    dbc = _dbc(dbc, len(d_x), y.shape[-1])
    return derivative(y[..., 1:2], d_x[0], 0, dbc[0, 1:2]) - derivative(
        y[..., :1], d_x[1], 1, dbc[1, :1]
    )


# ------------------------------------------------ curvilinear operators
# numerical_differentiator.py restated for POLAR (r, theta), CYLINDRICAL
# (r, theta, z) and SPHERICAL (r, theta, phi) meshes: each operator is the
# Cartesian discrete derivative(s) above scaled by the vertex coordinates,
# in the reference's own order of operations.
def gradient_cs(cs, y, d_x, axis, dbc, grids):
    """numerical_differentiator.py:114-156."""
    dbc = _dbc(dbc, len(d_x), y.shape[-1])
    d = derivative(y, d_x[axis], axis, dbc[axis])
    if cs == "SPHERICAL":
        r = grids[0][..., np.newaxis]
        phi = grids[2][..., np.newaxis]
        if axis == 0:
            return d
        if axis == 1:
            return d / (r * np.sin(phi))
        return d / r
    if axis == 1:
        return d / grids[0][..., np.newaxis]
    return d


def hessian_cs(cs, y, d_x, a1, a2, dbc, grids):
    """numerical_differentiator.py:175-308."""
    dbc = _dbc(dbc, len(d_x), y.shape[-1])
    sd = second_derivative(y, d_x[a1], d_x[a2], a1, a2, dbc[a1])
    r = grids[0][..., np.newaxis]
    dr = lambda: derivative(y, d_x[0], 0, dbc[0])  # noqa: E731
    if cs == "SPHERICAL":
        phi = grids[2][..., np.newaxis]
        if a1 == 0 and a2 == 0:
            return sd
        if a1 == 1 and a2 == 1:
            sin_phi, cos_phi = np.sin(phi), np.cos(phi)
            d_phi = derivative(y, d_x[2], 2, dbc[2])
            return (dr() + (sd / sin_phi + cos_phi * d_phi) / (r * sin_phi)) / r
        if a1 == 2 and a2 == 2:
            return (sd / r + dr()) / r
        if {a1, a2} == {0, 1}:
            d_theta = derivative(y, d_x[1], 1, dbc[1])
            return (sd - d_theta / r) / (r * np.sin(phi))
        if {a1, a2} == {0, 2}:
            d_phi = derivative(y, d_x[2], 2, dbc[2])
            return (sd - d_phi / r) / r
        sin_phi, cos_phi = np.sin(phi), np.cos(phi)
        d_theta = derivative(y, d_x[1], 1, dbc[1])
        return (sin_phi * sd - cos_phi * d_theta) / (r * sin_phi) ** 2
    if a1 in (0, 2) and a2 in (0, 2):
        return sd
    if a1 == 1 and a2 == 1:
        return (sd / r + dr()) / r
    if {a1, a2} == {0, 1}:
        d_theta = derivative(y, d_x[1], 1, dbc[1])
        return (sd - d_theta / r) / r
    return sd / r


def laplacian_cs(cs, y, d_x, dbc, grids):
    """numerical_differentiator.py:592-725."""
    dbc = _dbc(dbc, len(d_x), y.shape[-1])
    r = grids[0][..., np.newaxis]
    d_r = derivative(y, d_x[0], 0, dbc[0])
    sd_r = second_derivative(y, d_x[0], d_x[0], 0, 0, dbc[0])
    sd_theta = second_derivative(y, d_x[1], d_x[1], 1, 1, dbc[1])
    if cs == "SPHERICAL":
        phi = grids[2][..., np.newaxis]
        sin_phi, cos_phi = np.sin(phi), np.cos(phi)
        d_phi = derivative(y, d_x[2], 2, dbc[2])
        sd_phi = second_derivative(y, d_x[2], d_x[2], 2, 2, dbc[2])
        return sd_r + (2 * d_r + (sd_phi + (cos_phi * d_phi + sd_theta / sin_phi) / sin_phi) / r) / r
    lap = sd_r + (sd_theta / r + d_r) / r
    if cs == "POLAR":
        return lap
    return lap + second_derivative(y, d_x[2], d_x[2], 2, 2, dbc[2])


def divergence_cs(cs, y, d_x, dbc, grids):
    """numerical_differentiator.py:310-400."""
    dbc = _dbc(dbc, len(d_x), y.shape[-1])
    r = grids[0][..., np.newaxis]
    y_r, y_theta = y[..., :1], y[..., 1:2]
    d_r = derivative(y_r, d_x[0], 0, dbc[0, :1])
    d_theta = derivative(y_theta, d_x[1], 1, dbc[1, 1:2])
    if cs == "SPHERICAL":
        phi = grids[2][..., np.newaxis]
        sin_phi, cos_phi = np.sin(phi), np.cos(phi)
        y_phi = y[..., 2:]
        d_phi = derivative(y_phi, d_x[2], 2, dbc[2, 2:])
        return d_r + (d_phi + 2.0 * y_r + (d_theta + cos_phi * y_phi) / sin_phi) / r
    div = d_r + (y_r + d_theta) / r
    if cs == "POLAR":
        return div
    return div + derivative(y[..., 2:], d_x[2], 2, dbc[2, 2:])


def curl_cs(cs, y, d_x, curl_ind, dbc, grids):
    """numerical_differentiator.py:402-590 (CARTESIAN 3D included)."""
    dbc = _dbc(dbc, len(d_x), y.shape[-1])
    if cs == "CARTESIAN":
        if len(d_x) == 2 or curl_ind == 2:
            return derivative(y[..., 1:2], d_x[0], 0, dbc[0, 1:2]) - derivative(y[..., :1], d_x[1], 1, dbc[1, :1])
        if curl_ind == 0:
            return derivative(y[..., 2:], d_x[1], 1, dbc[1, 2:]) - derivative(y[..., 1:2], d_x[2], 2, dbc[2, 1:2])
        return derivative(y[..., :1], d_x[2], 2, dbc[2, :1]) - derivative(y[..., 2:], d_x[0], 0, dbc[0, 2:])
    r = grids[0][..., np.newaxis]
    if cs == "SPHERICAL":
        if curl_ind == 0:
            phi = grids[2][..., np.newaxis]
            sin_phi, cos_phi = np.sin(phi), np.cos(phi)
            y_theta, y_phi = y[..., 1:2], y[..., 2:]
            d_theta_phi = derivative(y_theta, d_x[2], 2, dbc[2, 1:2])
            d_phi_theta = derivative(y_phi, d_x[1], 1, dbc[1, 2:])
            return (d_theta_phi + (cos_phi * y_theta - d_phi_theta) / sin_phi) / r
        if curl_ind == 1:
            y_r, y_phi = y[..., :1], y[..., 2:]
            d_r_phi = derivative(y_r, d_x[2], 2, dbc[2, :1])
            d_phi_r = derivative(y_phi, d_x[0], 0, dbc[0, 2:])
            return d_phi_r + (y_phi - d_r_phi) / r
        sin_phi = np.sin(grids[2][..., np.newaxis])
        y_r, y_theta = y[..., :1], y[..., 1:2]
        d_r_theta = derivative(y_r, d_x[1], 1, dbc[1, :1])
        d_theta_r = derivative(y_theta, d_x[0], 0, dbc[0, 1:2])
        return -d_theta_r + (d_r_theta / sin_phi - y_theta) / r
    if cs == "POLAR" or curl_ind == 2:
        y_r, y_theta = y[..., :1], y[..., 1:2]
        d_r_theta = derivative(y_r, d_x[1], 1, dbc[1, :1])
        d_theta_r = derivative(y_theta, d_x[0], 0, dbc[0, 1:2])
        return d_theta_r + (y_theta - d_r_theta) / r
    if curl_ind == 0:
        d_z_theta = derivative(y[..., 2:], d_x[1], 1, dbc[1, 2:])
        d_theta_z = derivative(y[..., 1:2], d_x[2], 2, dbc[2, 1:2])
        return d_z_theta / r - d_theta_z
    d_r_z = derivative(y[..., :1], d_x[2], 2, dbc[2, :1])
    d_z_r = derivative(y[..., 2:], d_x[0], 0, dbc[0, 2:])
    return d_r_z - d_z_r


def implicit_integral(y, t: float, d_t: float, f, c, a: float = 1.0, crank_nicolson: bool = False,
                      tol: float = 1.48e-8, maxiter: int = 50):
    """BackwardEulerMethod / CrankNicolsonMethod.integral
    (numerical_integrator.py:199-270) on any right-hand side f(t, y) and
    constraint function c(t): forward Euler predictor, then the secant solve
    of y_next - c(t + dt)(y + a dt f(t + dt, y_next) + (1 - a) dt f(t, y)).
    Returns (y_next, secant iterations, warning or None)."""
    t_next = t + d_t
    c_next = c(t_next)
    forward = d_t * f(t, y)
    init = apply_y_constraints(c_next, y + forward)
    if not crank_nicolson:
        def residual(x):
            return x - apply_y_constraints(c_next, y + d_t * f(t_next, x))
    else:
        b = 1.0 - a

        def residual(x):
            return x - apply_y_constraints(c_next, y + a * d_t * f(t_next, x) + b * forward)
    return secant_solve(residual, init, tol, maxiter)


# ---------------------------------------------------------------- Jacobi
def anti_laplacian_estimate(cs, y_hat, lap, d_x, dbc, grids) -> np.ndarray:
    """One Jacobi update of the Poisson estimate y_hat (every coordinate system)."""
    if not np.all(np.array(y_hat.shape[:-1]) > 2):
        raise ValueError("y must contain at least 3 points along all x axes")
    out = np.zeros_like(y_hat)
    all_d_x_sqr = np.square(d_x)
    r = r_sqr = phi = sin_phi = r_sqr_sin_phi_sqr = None
    if cs != "CARTESIAN":
        r = grids[0][..., np.newaxis]
        r_sqr = r**2
        if cs == "SPHERICAL":
            phi = grids[2][..., np.newaxis]
            sin_phi = np.sin(phi)
            r_sqr_sin_phi_sqr = r_sqr * sin_phi**2
    sl = [slice(None)] * y_hat.ndim
    for axis, h in enumerate(d_x):
        ext = _halos(y_hat, axis, h, dbc[axis])
        sl[axis] = slice(0, -2)
        prev = ext[tuple(sl)]
        sl[axis] = slice(2, None)
        nxt = ext[tuple(sl)]
        sl[axis] = slice(None)
        upd = (prev + nxt) / all_d_x_sqr[axis]
        if cs == "CARTESIAN":
            out += upd
        elif cs == "SPHERICAL":
            if axis == 0:
                out += upd + (nxt - prev) / (h * r)
            elif axis == 1:
                out += upd / r_sqr_sin_phi_sqr
            else:
                out += (upd + np.cos(phi) * (nxt - prev) / (2.0 * h * sin_phi)) / r_sqr
        else:
            if axis == 0:
                out += upd + (nxt - prev) / (2.0 * h * r)
            elif axis == 1:
                out += upd / r_sqr
            else:
                out += upd
    out -= lap
    if cs == "CARTESIAN":
        return out / (2.0 / all_d_x_sqr).sum()
    if cs == "SPHERICAL":
        return out / (2.0 / all_d_x_sqr[0] + 2.0 / (all_d_x_sqr[1] * r_sqr_sin_phi_sqr)
                      + 2.0 / (all_d_x_sqr[2] * r_sqr))
    step = 2.0 / all_d_x_sqr[0] + 2.0 / (all_d_x_sqr[1] * r_sqr)
    if cs == "POLAR":
        return out / step
    return out / (step + 2.0 / all_d_x_sqr[2])


def anti_laplacian(cs, lap, d_x, y_constraints, dbc, grids, tol: float, y_init=None,
                   counter: Optional[list] = None) -> np.ndarray:
    """Jacobi solve of lap(y) = ``lap``: start from ``y_init`` (else
    ``np.random.random``, the reference's estimate), constrained; iterate
    while the 2-norm of the change exceeds tol.  ``counter`` (a list)
    receives the iteration count."""
    dbc = _dbc(dbc, len(d_x), lap.shape[-1])
    y = np.random.random(lap.shape) if y_init is None else np.array(y_init, dtype=np.float64)
    apply_y_constraints(y_constraints, y)
    diff, it = np.inf, 0
    while diff > tol:
        y_old = y
        y = anti_laplacian_estimate(cs, y_old, lap, d_x, dbc, grids)
        apply_y_constraints(y_constraints, y)
        diff = float(np.linalg.norm(y - y_old))
        it += 1
    if counter is not None:
        counter.append(it)
    return y


# ---------------------------------------------------------------- RHS
class RHS:
    """Symbol map + lambdified right-hand sides (symbol_mapper.py:160-271)."""

    def __init__(self, cp):
        self.cp = cp
        de = cp.differential_equation
        eq = de.symbolic_equation_system
        self.rhs = list(eq.rhs)
        kinds = [int(getattr(k, "value", k)) for k in eq.lhs_types]
        self.d_idx = [i for i, k in enumerate(kinds) if k == 0]
        self.y_idx = [i for i, k in enumerate(kinds) if k == 1]
        self.lap_idx = [i for i, k in enumerate(kinds) if k == 2]
        self.d_x = tuple(cp.mesh.d_x) if de.x_dimension else ()
        self.grids = cp.mesh.vertex_coordinate_grids if de.x_dimension else ()
        cst = cp.mesh.coordinate_system_type if de.x_dimension else None
        self.cs = getattr(cst, "name", str(cst)) if cst is not None else "CARTESIAN"
        self._fns = {}
        for name, rows in (("d", self.d_idx), ("y", self.y_idx), ("l", self.lap_idx)):
            if not rows:
                continue
            syms = list(set().union(*[self.rhs[i].free_symbols for i in rows]))
            fn = sp.lambdify([syms], [self.rhs[i] for i in rows], "numpy")
            self._fns[name] = (syms, fn)

    def _value(self, sym, t, y, dbc):
        tokens = sym.name.split("_")
        prefix, idx = tokens[0], [int(k) for k in tokens[1:]]
        if prefix == "t":
            return np.array([t])
        if prefix == "y":
            return y[..., idx[0]: idx[0] + 1]
        if prefix == "x":
            return self.grids[idx[0]][..., np.newaxis]
        sub = lambda ind: dbc[:, ind] if dbc is not None else None  # noqa: E731
        if self.cs != "CARTESIAN":
            g = self.grids
            if prefix == "y-gradient":
                i, j = idx
                return gradient_cs(self.cs, y[..., i: i + 1], self.d_x, j, sub(slice(i, i + 1)), g)
            if prefix == "y-hessian":
                i, j, k = idx
                return hessian_cs(self.cs, y[..., i: i + 1], self.d_x, j, k, sub(slice(i, i + 1)), g)
            if prefix == "y-laplacian":
                i = idx[0]
                return laplacian_cs(self.cs, y[..., i: i + 1], self.d_x, sub(slice(i, i + 1)), g)
            if prefix == "y-divergence":
                return divergence_cs(self.cs, y[..., idx], self.d_x, sub(idx), g)
            if prefix == "y-curl":
                return curl_cs(self.cs, y[..., idx[:-1]], self.d_x, idx[-1], sub(idx[:-1]), g)
            raise KeyError(sym)
        if prefix == "y-gradient":
            i, j = idx
            return gradient(y[..., i: i + 1], self.d_x, j, dbc[:, i: i + 1] if dbc is not None else None)
        if prefix == "y-hessian":
            i, j, k = idx
            return hessian(y[..., i: i + 1], self.d_x, j, k, dbc[:, i: i + 1] if dbc is not None else None)
        if prefix == "y-laplacian":
            i = idx[0]
            return laplacian(y[..., i: i + 1], self.d_x, dbc[:, i: i + 1] if dbc is not None else None)
        if prefix == "y-divergence":
            return divergence(y[..., idx], self.d_x, dbc[:, idx] if dbc is not None else None)
        if prefix == "y-curl":
            if len(idx) == 4:  # 3D: three y indices and the curl component
                return curl_cs("CARTESIAN", y[..., idx[:3]], self.d_x, idx[3], sub(idx[:3]), self.grids)
            return curl2d(y[..., idx], self.d_x, dbc[:, idx] if dbc is not None else None)
        raise KeyError(sym)

    def evaluate(self, which: str, t: float, y: np.ndarray, dbc) -> np.ndarray:
        syms, fn = self._fns[which]
        vals = fn([self._value(s, t, y, dbc) for s in syms])
        shape = y.shape[:-1] + (1,)
        return np.concatenate([np.broadcast_to(v, shape) for v in vals], axis=-1)


# ---------------------------------------------------------------- stepping
class FDMStepper:
    """y(t) -> y(t + d_t) exactly as FDMOperator's y_next_function."""

    def __init__(self, cp, integrator: str, d_t: float, tol: float = 1e-3, secant_tol: float = 1.48e-8,
                 secant_maxiter: int = 50, cn_a: float = 0.5):
        if integrator not in (FE, MIDPOINT, RK4, BACKWARD_EULER, CRANK_NICOLSON):
            raise ValueError(integrator)
        self.tol = tol  # Jacobi tolerance of the LHS.Y_LAPLACIAN solves
        self.secant_tol, self.secant_maxiter, self.cn_a = secant_tol, secant_maxiter, cn_a
        self.secant_iterations: List[int] = []
        self.jacobi_iterations: List[int] = []
        self.cp = cp
        self.integrator = integrator
        self.d_t = d_t
        self.rhs = RHS(cp)
        x_dim = cp.differential_equation.x_dimension
        self.dynamic = bool(x_dim) and not cp.are_all_boundary_conditions_static
        self.y_c = cp.static_y_vertex_constraints if x_dim else None
        self.dy_c = cp.static_boundary_vertex_constraints[1] if x_dim else None

    # time-dependent conditions: the reference's constraint functions
    # (fdm_operator.py:199-231) re-create the constraints for each time
    def yc(self, t: float):
        if not self.dynamic:
            return self.y_c
        return self.cp.create_y_vertex_constraints(self.cp.create_boundary_constraints(True, t)[0])

    def dyc(self, t: float):
        if not self.dynamic:
            return self.dy_c
        return self.cp.create_boundary_constraints(True, t)[1]

    def f(self, t: float, y: np.ndarray) -> np.ndarray:
        out = np.zeros(y.shape)
        out[..., self.rhs.d_idx] = self.rhs.evaluate("d", t, y, self.dyc(t))
        return out

    def step(self, t: float, y: np.ndarray) -> np.ndarray:
        """RK4/midpoint/FE as numerical_integrator.py:42-132: every stage
        input constrained at its own time, the result at t + d_t."""
        d_t, f, c = self.d_t, self.f, self.yc
        if self.integrator in (BACKWARD_EULER, CRANK_NICOLSON):
            cn = self.integrator == CRANK_NICOLSON
            y_next, its, warning = implicit_integral(y, t, d_t, f, c, self.cn_a if cn else 1.0, cn,
                                                     self.secant_tol, self.secant_maxiter)
            if warning is not None:  # scipy.optimize.newton warns the same way
                import warnings

                warnings.warn(warning, RuntimeWarning, stacklevel=2)
            self.secant_iterations.append(its)
        elif self.integrator == FE:
            y_next = apply_y_constraints(c(t + d_t), y + d_t * f(t, y))
        elif self.integrator == MIDPOINT:
            h = d_t / 2.0
            y_hat = apply_y_constraints(c(t + h), y + h * f(t, y))
            y_next = apply_y_constraints(c(t + d_t), y + d_t * f(t + h, y_hat))
        else:
            h = d_t / 2.0
            k1 = d_t * f(t, y)
            k2 = d_t * f(t + h, apply_y_constraints(c(t + h), y + k1 / 2.0))
            k3 = d_t * f(t + h, apply_y_constraints(c(t + h), y + k2 / 2.0))
            k4 = d_t * f(t + d_t, apply_y_constraints(c(t + d_t), y + k3))
            y_next = apply_y_constraints(c(t + d_t), y + (k1 + 2.0 * k2 + 2.0 * k3 + k4) / 6.0)
        if self.rhs.y_idx:
            y_rhs = self.rhs.evaluate("y", t, y, self.dyc(t))
            c_end = c(t + d_t)
            sub = None if c_end is None else c_end[self.rhs.y_idx]
            y_next[..., self.rhs.y_idx] = apply_y_constraints(sub, y_rhs)
        if self.rhs.lap_idx:  # fdm_operator.py:141-161
            lap = self.rhs.evaluate("l", t, y, self.dyc(t))
            c_end, dc_end = c(t + d_t), self.dyc(t + d_t)
            sub = None if c_end is None else c_end[self.rhs.lap_idx]
            dsub = None if dc_end is None else dc_end[:, self.rhs.lap_idx]
            y_next[..., self.rhs.lap_idx] = anti_laplacian(
                self.rhs.cs, lap, self.rhs.d_x, sub, dsub, self.rhs.grids, self.tol,
                counter=self.jacobi_iterations)
        return y_next


def time_grid(t_interval, d_t: float) -> np.ndarray:
    """discretize_time_domain (operator.py:60-74)."""
    t0 = t_interval[0]
    steps = int(round((t_interval[1] - t0) / d_t))
    return np.linspace(t0, t0 + steps * d_t, steps + 1)


def fdm_solve(
    cp,
    y0: np.ndarray,
    t_interval,
    d_t: float,
    integrator: str,
    keep: str = "full",
    n_steps: Optional[int] = None,
    tol: float = 1e-3,
    **stepper_kw,
) -> np.ndarray:
    """Trajectory y[1..n] (keep='full') or the final state (keep='final');
    ``stepper_kw``: secant settings of the implicit integrators."""
    stepper = FDMStepper(cp, integrator, d_t, tol, **stepper_kw)
    t = time_grid(t_interval, d_t)
    steps = len(t) - 1 if n_steps is None else n_steps
    y = np.array(y0, dtype=np.float64, copy=True)
    if stepper.dynamic:  # fdm_operator.py:56-63: constrain the initial state at t0
        y = apply_y_constraints(stepper.yc(t[0]), y)
    traj = [] if keep == "full" else None
    for i in range(steps):
        y = stepper.step(t[i], y)
        if traj is not None:
            traj.append(y)
    return np.stack(traj) if traj is not None else y


def rms_update_norms(old: np.ndarray, new: np.ndarray) -> np.ndarray:
    """Per-component max over slices of the RMS update (parareal_operator.py:85-100)."""
    y_dim = old.shape[-1]
    out = np.empty(y_dim)
    for k in range(y_dim):
        best = 0.0
        for n_j, o_j in zip(new[..., k], old[..., k]):
            best = np.maximum(best, np.sqrt(np.square(n_j - o_j).mean()))
        out[k] = best
    return out


def parareal_solve(
    cp,
    y0: np.ndarray,
    t_interval,
    n_slices: int,
    fine: Callable[[np.ndarray, float, float], np.ndarray],
    coarse: Callable[[np.ndarray, float, float], np.ndarray],
    tol,
    max_iterations: int,
    fine_traj: Optional[Callable[[np.ndarray, float, float], np.ndarray]] = None,
):
    """Serial replay of PararealOperator.solve (parareal_operator.py:102-197).

    ``fine``/``coarse`` map (y_start, t_start, t_end) to the end state of one
    slice; ``fine_traj`` (optional) returns the whole fine sub-trajectory.
    Returns (border points U[0..S], iterations, fine trajectory or None).
    """
    borders = np.linspace(t_interval[0], t_interval[1], n_slices + 1)
    coarse_ends = []
    y = y0
    for j in range(n_slices):
        y = coarse(y, borders[j], borders[j + 1])
        coarse_ends.append(y)
    coarse_ends = np.stack(coarse_ends)
    u = np.concatenate([y0[np.newaxis], coarse_ends])
    y_dim = y0.shape[-1]
    tols = np.array(tol if isinstance(tol, (list, tuple, np.ndarray)) else [tol] * y_dim)
    iterations = 0
    start_points = None
    for i in range(min(n_slices, max_iterations)):
        start_points = u.copy()
        fine_ends = np.stack([fine(u[j], borders[j], borders[j + 1]) for j in range(n_slices)])
        corrections = fine_ends - coarse_ends
        old = u[1:].copy()
        for j in range(i, n_slices):
            if j > i:
                coarse_ends[j] = coarse(u[j], borders[j], borders[j + 1])
            u[j + 1] = coarse_ends[j] + corrections[j]
        iterations = i + 1
        if np.all(rms_update_norms(old, u[1:]) < tols):
            break
    traj = None
    if fine_traj is not None:
        parts = []
        for j in range(n_slices):
            sub = fine_traj(start_points[j], borders[j], borders[j + 1])
            parts.append(sub + (u[j + 1] - sub[-1]))
        traj = np.concatenate(parts)
    return u, iterations, traj
