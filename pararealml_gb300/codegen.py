"""Lowering of constrained problems and CUDA code generation.

``lower_problem`` turns a constrained problem (this package's or the
reference's own ``ConstrainedProblem`` object: only its public attributes are
read) into a ``LoweredProblem``: kernel-axis geometry, dense NaN-masked
Dirichlet / Neumann face tables built from
``static_boundary_vertex_constraints`` (reference
``constrained_problem.py:303-476``) and the symbolic right-hand sides.

``generate_source`` prints those right-hand sides as CUDA C++ device code
(the GPU counterpart of ``sympy.lambdify`` in ``symbol_mapper.py:246``) and
instantiates the fused step kernels of ``csrc/fdm_step.cuh``.  The symbol
grammar is the reference's (``symbol_mapper.py:160-220``): ``t``, ``y_i``,
``x_j``, ``y-gradient_i_j``, ``y-hessian_i_j_k``, ``y-laplacian_i``,
``y-divergence_i..``, ``y-curl_i..``.  Float constants are printed with
sympy's own numeric printer so that the kernel multiplies by exactly the
doubles that the reference's lambdified numpy code uses.
"""

from __future__ import annotations

import dataclasses
import hashlib
from typing import Dict, List, Sequence, Tuple

import numpy as np
import sympy as sp
from sympy.printing.c import C99CodePrinter
from sympy.printing.numpy import NumPyPrinter

# integrator kinds (number of stages), matching prml::Integrator
FORWARD_EULER = 1
EXPLICIT_MIDPOINT = 2
# implicit integrators: no stage schedule of their own (each step is a
# secant solve over right-hand-side evaluations)
BACKWARD_EULER = 8
CRANK_NICOLSON = 9
IMPLICIT = (BACKWARD_EULER, CRANK_NICOLSON)
RK4 = 4

LHS_D_Y_OVER_D_T = 0
LHS_Y = 1
LHS_Y_LAPLACIAN = 2

# candidate CTA tiles (rows, cols, threads) tried by the autotuner
TILE_CONFIGS: Tuple[Tuple[int, int, int], ...] = (
    (32, 32, 256),
    (16, 64, 256),
    (32, 64, 256),
    (16, 32, 128),
    (8, 64, 128),
    (16, 32, 256),
    (32, 32, 128),
    (16, 64, 128),
)
# temporally blocked variants (rows, cols, threads, steps per launch), built
# for single-stage steps only (forward Euler, or stage-invariant systems)
TB_CONFIGS: Tuple[Tuple[int, int, int, int], ...] = tuple(
    tile + (k,) for tile in ((16, 32, 128), (32, 32, 256), (32, 64, 256)) for k in (2, 4, 8)
)
# register-window kernels (walk_body) for single-stage steps on 2D meshes:
# (rows per thread R, warps per CTA); the tile is 4 R rows by 8 warps x 16
# bytes of columns, keyed (4 R, cols, threads, 1, 0, "w")
WALK_CONFIGS: Tuple[Tuple[int, int], ...] = ((1, 4), (2, 2), (2, 4), (4, 2), (4, 4))
# 3D tiles (rows, cols, threads, 1, planes)
TILE_CONFIGS_3D: Tuple[Tuple[int, int, int, int, int], ...] = (
    (8, 32, 256, 1, 2),
    (4, 32, 256, 1, 4),
    (4, 32, 128, 1, 2),
    (8, 32, 256, 1, 4),
    (8, 32, 256, 1, 1),
    (4, 16, 128, 1, 2),
    (2, 16, 64, 1, 2),
)
SMEM_LIMIT = 227 * 1024
# tiles of the multi-round kernels (one cooperative launch takes every step
# of several groups of instances, a grid barrier between rounds)
MULTI_TILES: Tuple[Tuple[int, int, int], ...] = ((16, 32, 256), (32, 32, 256), (16, 64, 256), (16, 32, 128), (8, 64, 128))
# static shared memory of a multi-round kernel besides its dynamic buffers
# (the groups' launch parameters and round tables)
MULTI_STATIC_SMEM = 8 * 512 + 128


@dataclasses.dataclass
class LoweredProblem:
    x_dimension: int
    vertices_shape: Tuple[int, ...]
    n_comp: int
    nx: int
    ny: int
    kaxis: Tuple[int, ...]  # mesh axis -> kernel axis
    dx_k: Tuple[float, float]  # step size per kernel axis (1.0 if unused)
    d_idx: Tuple[int, ...]
    y_idx: Tuple[int, ...]
    rhs: Tuple[sp.Expr, ...]
    dirichlet: np.ndarray  # (4, C, face_len) float64, NaN = free
    neumann: np.ndarray
    dir_mask: int
    neu_mask: int
    coord_k0: np.ndarray
    coord_k1: np.ndarray
    # time-dependent boundary conditions: the tables above are placeholders
    # and face_tables_at(low, t) evaluates them per time
    dynamic: bool = False
    cp: object = None
    # 3D meshes: planes along mesh axis 0 (kernel axis 0); rows / columns
    # above are mesh axes 1 and 2
    nz: int = 1
    dx_z: float = 1.0
    coord_kz: np.ndarray = None
    # coordinate system of the mesh: CARTESIAN, POLAR (r, theta),
    # CYLINDRICAL (r, theta, z) or SPHERICAL (r, theta, phi)
    cs: str = "CARTESIAN"
    # components with LHS.Y_LAPLACIAN (solved by Jacobi after each step)
    lap_idx: Tuple[int, ...] = ()
    # step sizes and vertex coordinates per mesh axis (reference order)
    mesh_dx: Tuple[float, ...] = ()
    axis_coords: Tuple[np.ndarray, ...] = ()

    @property
    def face_len(self) -> int:
        return self.dirichlet.shape[-1]


def _lhs_value(kind) -> int:
    return int(getattr(kind, "value", kind))


def _dense(constraint) -> np.ndarray:
    mask = np.asarray(constraint.mask)
    out = np.full(mask.shape, np.nan)
    out[mask] = np.asarray(constraint.values).reshape(-1)
    return out.reshape(-1)


def lower_problem(cp) -> LoweredProblem:
    """Reads the static description of a constrained problem."""
    diff_eq = cp.differential_equation
    x_dim = diff_eq.x_dimension
    n_comp = diff_eq.y_dimension
    eq_sys = diff_eq.symbolic_equation_system
    kinds = [_lhs_value(k) for k in eq_sys.lhs_types]
    if n_comp > 16 or (x_dim == 3 and n_comp > 10):
        raise NotImplementedError("at most 16 solution components (10 on 3D meshes) are supported")
    if x_dim > 3:
        raise NotImplementedError("the GPU FDM path supports 0 to 3 spatial dimensions")
    if x_dim:
        mesh = cp.mesh
        cs = getattr(mesh.coordinate_system_type, "name", str(mesh.coordinate_system_type))
        if cs not in ("CARTESIAN", "POLAR", "CYLINDRICAL", "SPHERICAL"):
            raise NotImplementedError(f"unsupported coordinate system {cs}")
        shape = tuple(int(n) for n in mesh.vertices_shape)
        d_x = tuple(float(h) for h in mesh.d_x)
    else:
        shape = ()
        d_x = ()

    nz, dx_z, coord_kz = 1, 1.0, np.zeros(1)
    if x_dim == 3:
        kaxis = (0, 1, 2)
        nz, nx, ny = shape
        dx_k = (d_x[1], d_x[2])
        dx_z = d_x[0]
        coords = [np.asarray(c, dtype=np.float64) for c in cp.mesh.vertex_axis_coordinates]
        coord_kz, coord_k0, coord_k1 = coords[0], coords[1], coords[2]
    elif x_dim == 2:
        kaxis = (0, 1)
        nx, ny = shape
        dx_k = (d_x[0], d_x[1])
        coords = [np.asarray(c, dtype=np.float64) for c in cp.mesh.vertex_axis_coordinates]
        coord_k0, coord_k1 = coords[0], coords[1]
    elif x_dim == 1:
        kaxis = (1,)
        nx, ny = 1, shape[0]
        dx_k = (1.0, d_x[0])
        coord_k0 = np.zeros(1)
        coord_k1 = np.asarray(cp.mesh.vertex_axis_coordinates[0], dtype=np.float64)
    else:
        kaxis = ()
        nx = ny = 1
        dx_k = (1.0, 1.0)
        coord_k0 = np.zeros(1)
        coord_k1 = np.zeros(1)

    # a face of a 3D mesh is a plane, indexed in C order by the other axes
    face_len = max(nx, ny) if x_dim < 3 else max(nx * ny, nz * ny, nz * nx)
    n_faces = 6 if x_dim == 3 else 4
    dynamic = bool(x_dim) and not bool(cp.are_all_boundary_conditions_static)
    if x_dim and not dynamic:
        dirichlet, neumann, dir_mask, neu_mask = _face_tables(
            cp.static_boundary_vertex_constraints, x_dim, kaxis, n_comp, face_len, n_faces
        )
    else:
        dirichlet = np.full((n_faces, n_comp, face_len), np.nan)
        neumann = np.full((n_faces, n_comp, face_len), np.nan)
        dir_mask = neu_mask = 0
    if dynamic:
        # the kernel tests a face of a component only where its bit is set;
        # set it wherever a condition of that kind exists (NaN values at a
        # given time still mean "free")
        for axis, pair in enumerate(cp.boundary_conditions):
            for side, bc in enumerate(pair):
                face = 2 * kaxis[axis] + side
                for comp in range(n_comp):
                    bit = 1 << (face * n_comp + comp)
                    if bc.has_y_condition:
                        dir_mask |= bit
                    if bc.has_d_y_condition:
                        neu_mask |= bit

    d_idx = tuple(i for i, k in enumerate(kinds) if k == LHS_D_Y_OVER_D_T)
    # LHS.Y_LAPLACIAN rows: the step kernel stores their right-hand side at
    # (t, y) like an LHS.Y row, and the Jacobi solve replaces it with its
    # anti-Laplacian (fdm_operator.py:141-161).  The Dirichlet values the
    # store imposes only touch vertices whose solution value is overwritten
    # by the same values in every Jacobi iteration, so the right-hand side
    # there is never read.
    lap_idx = tuple(i for i, k in enumerate(kinds) if k == LHS_Y_LAPLACIAN)
    if lap_idx and not x_dim:
        raise NotImplementedError("LHS.Y_LAPLACIAN needs a spatial mesh")
    y_idx = tuple(i for i, k in enumerate(kinds) if k in (LHS_Y, LHS_Y_LAPLACIAN))
    return LoweredProblem(
        x_dimension=x_dim,
        vertices_shape=shape,
        n_comp=n_comp,
        nx=nx,
        ny=ny,
        kaxis=kaxis,
        dx_k=dx_k,
        d_idx=d_idx,
        y_idx=y_idx,
        rhs=tuple(eq_sys.rhs),
        dirichlet=dirichlet,
        neumann=neumann,
        dir_mask=dir_mask,
        neu_mask=neu_mask,
        coord_k0=coord_k0,
        coord_k1=coord_k1,
        dynamic=dynamic,
        cp=cp if dynamic else None,
        nz=nz,
        dx_z=dx_z,
        coord_kz=coord_kz,
        cs=cs if x_dim else "CARTESIAN",
        lap_idx=lap_idx,
        mesh_dx=d_x,
        axis_coords=tuple(np.asarray(c, dtype=np.float64) for c in cp.mesh.vertex_axis_coordinates) if x_dim else (),
    )


def _face_tables(pairs, x_dim, kaxis, n_comp, face_len, n_faces=4):
    """Dense (faces, C, face_len) Dirichlet and Neumann tables (NaN = free)
    and their presence bits from ``(y, dy/dn)`` boundary constraint pairs."""
    y_pairs, d_y_pairs = pairs
    dirichlet = np.full((n_faces, n_comp, face_len), np.nan)
    neumann = np.full((n_faces, n_comp, face_len), np.nan)
    dir_mask = neu_mask = 0
    for axis in range(x_dim):
        ka = kaxis[axis]
        for comp in range(n_comp):
            for table, tab_pairs, is_dir in ((dirichlet, y_pairs, True), (neumann, d_y_pairs, False)):
                pair = tab_pairs[axis, comp]
                if pair is None:
                    continue
                for side in (0, 1):
                    c = pair[side]
                    if c is None:
                        continue
                    vals = _dense(c)
                    face = 2 * ka + side
                    table[face, comp, : len(vals)] = vals
                    if np.any(~np.isnan(vals)):
                        bit = 1 << (face * n_comp + comp)
                        if is_dir:
                            dir_mask |= bit
                        else:
                            neu_mask |= bit
    return dirichlet, neumann, dir_mask, neu_mask


def face_tables_at(low: "LoweredProblem", t: float):
    """Face tables of a problem with time-dependent boundary conditions at
    time t: the reference re-creates its boundary constraints for every time
    it needs (``fdm_operator.py:199-231``, ``constrained_problem.py:303-348``)."""
    d, n, _, _ = _face_tables(low.cp.create_boundary_constraints(True, t), low.x_dimension, low.kaxis,
                              low.n_comp, low.face_len, low.dirichlet.shape[0])
    return d, n


# --------------------------------------------------------------------------
# symbols -> stencil calls


def _parse(symbol: sp.Symbol) -> Tuple[str, List[int]]:
    tokens = symbol.name.split("_")
    return tokens[0], [int(t) for t in tokens[1:]]


def _depends_on(symbols, comps: Sequence[int], with_t: bool) -> bool:
    comps = set(comps)
    for s in symbols:
        prefix, idx = _parse(s)
        if prefix == "t":
            if with_t:
                return True
        elif prefix == "x":
            continue
        elif prefix in ("y", "y-gradient", "y-hessian", "y-laplacian"):
            if idx[0] in comps:
                return True
        elif any(i in comps for i in idx):  # divergence, curl, vector Laplacian
            return True
    return False


def is_stage_invariant(low: LoweredProblem, integrator: int) -> bool:
    """True if dy/dt does not change across the integrator's stages.

    That is the case when the dy/dt right-hand sides read neither t nor any
    dy/dt component: stage inputs differ from y only in dy/dt components
    (reference ``fdm_operator.py:114-120``), so every stage evaluates the
    same function of the same values and k1 = k2 = k3 = k4 bit for bit.
    Cahn-Hilliard is such a system (dc/dt = d * lap(mu), mu has LHS.Y).
    """
    if integrator == FORWARD_EULER or low.dynamic:
        # time-dependent boundary values change the stage inputs and the
        # Neumann ghosts from stage to stage
        return False
    syms = set()
    for i in low.d_idx:
        syms |= low.rhs[i].free_symbols
    return not _depends_on(syms, low.d_idx, with_t=True)


def _symbol_code(sym: sp.Symbol, low: LoweredProblem, fast: bool = False) -> str:
    prefix, idx = _parse(sym)
    ka = low.kaxis
    x_dim = low.x_dimension

    def need3(axis: int):
        n = low.vertices_shape[axis]
        if n <= 2:
            raise ValueError(f"y must contain at least 3 points along x-axis ({axis})")

    if prefix == "t":
        return "a.t()"
    if prefix == "y":
        return f"a.template val<{idx[0]}>()"
    if prefix == "x":
        return f"a.template x<{ka[idx[0]]}>()"
    if low.cs != "CARTESIAN" and prefix in ("y-gradient", "y-hessian", "y-laplacian", "y-divergence", "y-curl"):
        for axis in range(x_dim):
            need3(axis)
        return _curvilinear_code(prefix, idx, low)
    if prefix == "y-gradient":
        i, j = idx
        need3(j)
        return f"a.template grad<{i}, {ka[j]}>()"
    if prefix == "y-hessian":
        i, j, k = idx
        need3(j)
        need3(k)
        return f"a.template hess<{i}, {ka[j]}, {ka[k]}>()"
    if prefix == "y-laplacian":
        i = idx[0]
        for axis in range(x_dim):
            need3(axis)
        if fast and x_dim == 2:
            return f"a.template lap<{i}>()"
        terms = [f"a.template sd<{i}, {ka[axis]}>()" for axis in range(x_dim)]
        return "(" + " + ".join(terms) + ")"
    if prefix == "y-divergence":
        if len(idx) != x_dim:
            raise ValueError("number of y indices of a divergence must match x dimensions")
        for axis in range(x_dim):
            need3(axis)
        terms = [f"a.template grad<{idx[axis]}, {ka[axis]}>()" for axis in range(x_dim)]
        return "(" + " + ".join(terms) + ")"
    if prefix == "y-curl":
        for axis in range(x_dim):
            need3(axis)
        if x_dim == 3 and len(idx) == 4:
            return _curvilinear_code(prefix, idx, low)
        if x_dim != 2:
            raise NotImplementedError("curl needs a 2D or 3D mesh")
        i0, i1 = idx[0], idx[1]
        return f"(a.template grad<{i1}, {ka[0]}>() - a.template grad<{i0}, {ka[1]}>())"
    if prefix == "y-vector-laplacian":
        # the reference never inserts these symbols into its symbol map
        # (symbol_mapper.py:215-218), so its FDM solver cannot evaluate them
        raise KeyError(sym)
    raise ValueError(f"unknown symbol {sym}")


def _curvilinear_code(prefix: str, idx, low: LoweredProblem) -> str:
    """Curvilinear operators (and the 3D Cartesian curl) as the reference's
    own expressions over the Cartesian discrete derivatives, operation for
    operation (operators/fdm/numerical_differentiator.py: gradient 114-156,
    hessian 175-308, divergence 310-400, curl 402-590, laplacian 592-725),
    with r = vertex coordinate of mesh axis 0 and phi that of axis 2."""
    ka, cs = low.kaxis, low.cs
    D = lambda c, a: f"a.template grad<{c}, {ka[a]}>()"  # noqa: E731  _derivative
    H = lambda c, a1, a2: f"a.template hess<{c}, {ka[a1]}, {ka[a2]}>()"  # noqa: E731  _second_derivative
    Y = lambda c: f"a.template val<{c}>()"  # noqa: E731
    R = f"a.template x<{ka[0]}>()"
    PHI = f"a.template x<{ka[2]}>()" if low.x_dimension == 3 else None
    SIN, COS = f"sin({PHI})", f"cos({PHI})"
    sph = cs == "SPHERICAL"
    if prefix == "y-gradient":
        c, ax = idx
        if sph:
            return D(c, ax) if ax == 0 else (f"({D(c, 1)} / ({R} * {SIN}))" if ax == 1 else f"({D(c, 2)} / {R})")
        return f"({D(c, 1)} / {R})" if ax == 1 else D(c, ax)
    if prefix == "y-hessian":
        c, a1, a2 = idx
        sd = H(c, a1, a2)
        pair = {a1, a2}
        if sph:
            if a1 == 0 and a2 == 0:
                return sd
            if a1 == 1 and a2 == 1:
                return f"(({D(c, 0)} + ((({sd} / {SIN}) + ({COS} * {D(c, 2)})) / ({R} * {SIN}))) / {R})"
            if a1 == 2 and a2 == 2:
                return f"((({sd} / {R}) + {D(c, 0)}) / {R})"
            if pair == {0, 1}:
                return f"(({sd} - ({D(c, 1)} / {R})) / ({R} * {SIN}))"
            if pair == {0, 2}:
                return f"(({sd} - ({D(c, 2)} / {R})) / {R})"
            return f"((({SIN} * {sd}) - ({COS} * {D(c, 1)})) / (({R} * {SIN}) * ({R} * {SIN})))"
        if a1 in (0, 2) and a2 in (0, 2):
            return sd
        if a1 == 1 and a2 == 1:
            return f"((({sd} / {R}) + {D(c, 0)}) / {R})"
        if pair == {0, 1}:
            return f"(({sd} - ({D(c, 1)} / {R})) / {R})"
        return f"({sd} / {R})"
    if prefix == "y-laplacian":
        c = idx[0]
        s0, s1 = H(c, 0, 0), H(c, 1, 1)
        if sph:
            s2 = H(c, 2, 2)
            return (f"({s0} + (((T(2) * {D(c, 0)}) + (({s2} + ((({COS} * {D(c, 2)}) + ({s1} / {SIN})) / {SIN}))"
                    f" / {R})) / {R}))")
        lap = f"({s0} + ((({s1} / {R}) + {D(c, 0)}) / {R}))"
        return lap if cs == "POLAR" else f"({lap} + {H(c, 2, 2)})"
    if prefix == "y-divergence":
        if len(idx) != low.x_dimension:
            raise ValueError("number of y indices of a divergence must match x dimensions")
        yr, yt = idx[0], idx[1]
        if sph:
            yp = idx[2]
            return (f"({D(yr, 0)} + ((({D(yp, 2)} + (T(2.0) * {Y(yr)})) + (({D(yt, 1)} + ({COS} * {Y(yp)})) / {SIN}))"
                    f" / {R}))")
        div = f"({D(yr, 0)} + (({Y(yr)} + {D(yt, 1)}) / {R}))"
        return div if cs == "POLAR" else f"({div} + {D(idx[2], 2)})"
    if prefix == "y-curl":
        if low.x_dimension != 3 or len(idx) != 4:
            raise NotImplementedError("curl on a curvilinear mesh needs a 3D vector field")
        i0, i1, i2, comp = idx
        if cs == "CARTESIAN":
            if comp == 2:
                return f"({D(i1, 0)} - {D(i0, 1)})"
            if comp == 0:
                return f"({D(i2, 1)} - {D(i1, 2)})"
            return f"({D(i0, 2)} - {D(i2, 0)})"
        if sph:
            if comp == 0:
                return f"(({D(i1, 2)} + ((({COS} * {Y(i1)}) - {D(i2, 1)}) / {SIN})) / {R})"
            if comp == 1:
                return f"({D(i2, 0)} + (({Y(i2)} - {D(i0, 2)}) / {R}))"
            return f"((-{D(i1, 0)}) + ((({D(i0, 1)} / {SIN}) - {Y(i1)}) / {R}))"
        if comp == 2:
            return f"({D(i1, 0)} + (({Y(i1)} - {D(i0, 1)}) / {R}))"
        if comp == 0:
            return f"(({D(i2, 1)} / {R}) - {D(i1, 2)})"
        return f"({D(i0, 2)} - {D(i2, 0)})"
    raise ValueError(prefix)


# Placeholder for the Laplacian's 1 / dx^2 in fused-order modules: the
# scaled Laplacian lap(y) is written lapr(y) * INV_DD, so that INV_DD joins
# the constant factors of its term (printed ``a.inv_dd()``).
INV_DD = sp.Symbol("__inv_dd")


def _is_const(factor) -> bool:
    """Whether a factor of a product is the same at every vertex and time
    (numbers and INV_DD): the printer groups such factors so that the
    compiler computes their product once per thread."""
    return bool(factor.is_number) or factor == INV_DD


def _const_split(term):
    """(constant factor, rest) of a product, or None when it has no
    constant factor or nothing else."""
    if not term.is_Mul:
        return None
    const = [f for f in term.args if _is_const(f)]
    var = [f for f in term.args if not _is_const(f)]
    if not const or not var:
        return None
    return sp.Mul(*const), sp.Mul(*var)


class _KernelPrinter(C99CodePrinter):
    """C99 printer emitting arithmetic in the kernel's real type ``T``."""

    def __init__(self, names: Dict[sp.Symbol, str], fast: bool = False):
        super().__init__()
        self._names = names
        self._num = NumPyPrinter()
        self._fast = fast

    def _fma_operands(self, term):
        """(rank, a, b) with term = a * b for a multiply-add, lower ranks
        first: a constant coefficient times the rest (the coefficient is
        computed once per thread), an integer power x^n = x^(n-1) * x, a
        product of variables (negated or not); a lone +-x last (a negation,
        free inside the multiply-add of the rest)."""
        split = _const_split(term)
        if split is not None:
            c, v = split
            if c in (1, -1):
                if v.is_Mul:
                    # +-(a b ...): a multiply-add with a negated factor (free)
                    a, b = v.as_two_terms()
                    return 2, (-a if c == -1 else a), b
                return 3, c, v  # +-x alone: a negation
            return 0, c, v
        if term.is_Pow and term.exp.is_Integer and int(term.exp) >= 2:
            return 1, sp.Pow(term.base, term.exp - 1), term.base
        if term.is_Mul:
            a, b = term.as_two_terms()
            return 2, a, b
        return None

    def _print_Add(self, expr):
        """Fused-order modules: a product term and the rest of the sum as
        one multiply-add (one rounding instead of two)."""
        if not self._fast:
            return super()._print_Add(expr)
        terms = list(self._as_ordered_terms(expr, order=None))
        best = None
        for k, term in enumerate(terms):
            ops = self._fma_operands(term)
            if ops is not None and (best is None or ops[0] < best[0]):
                best = (ops[0], k, ops[1], ops[2])
        if best is None or best[0] == 3:
            return super()._print_Add(expr)
        _, k, a, b = best
        rest = sp.Add(*(terms[:k] + terms[k + 1:]), evaluate=False)
        return f"prml::fmaT({self._print(a)}, {self._print(b)}, {self._print(rest)})"

    def _print_Mul(self, expr):
        """Fused-order modules: the constant factors of a product first and
        multiplied together, so the compiler computes them once per thread."""
        split = _const_split(expr) if self._fast else None
        if split is None or split[0] in (1, -1):
            return super()._print_Mul(expr)
        return f"({self._print(split[0])})*({self._print(split[1])})"

    def _print_Symbol(self, expr):
        return self._names[expr]

    def _print_Float(self, expr):
        return f"T({self._num.doprint(expr)})"

    def _print_Integer(self, expr):
        return f"T({int(expr)})"

    def _print_Rational(self, expr):
        return f"(T({int(expr.p)}) / T({int(expr.q)}))"

    def _print_NumberSymbol(self, expr):
        return f"T({repr(float(expr))})"

    _print_Pi = _print_NumberSymbol
    _print_Exp1 = _print_NumberSymbol

    def _print_Pow(self, expr):
        base, e = expr.base, expr.exp
        b = self.parenthesize(base, 1000)
        if e.is_Integer and 1 <= int(e) <= 8:
            return "(" + "*".join([b] * int(e)) + ")"
        if e.is_Integer and -8 <= int(e) <= -1:
            return "(T(1) / (" + "*".join([b] * (-int(e))) + "))"
        if e == sp.Rational(1, 2):
            return f"sqrt({self._print(base)})"
        return f"pow({self._print(base)}, {self._print(e)})"


def _folds_inv_dd(low: LoweredProblem, fast: bool) -> bool:
    """Fused-order 2D Cartesian modules with equal steps along both axes
    write scaled Laplacians as lapr(y) * INV_DD."""
    return fast and low.x_dimension == 2 and low.cs == "CARTESIAN" and low.dx_k[0] == low.dx_k[1]


def _rhs_function(name: str, rows: Sequence[int], low: LoweredProblem, fast: bool = False,
                  split: bool = False) -> str:
    """Device function ``name(a, f)`` setting f[k] to the right-hand side of
    row rows[k] at the vertex ``a``.  ``split``: ``name(a, f, fk)`` sets
    f[k] * fk[k] to it instead, fk[k] the product of the expression's
    constant factors (1 if it is not a product with one), for an update
    y + (dt fk[k]) f[k] with one multiply-add per vertex."""
    tail = ", typename P::real* fk" if split else ""
    if not rows:
        return (
            f"  template <class P> static __device__ __forceinline__ void {name}"
            f"(const P& a, typename P::real* f{tail}) {{ (void)a; (void)f; }}\n"
        )
    exprs = [low.rhs[i] for i in rows]
    syms = sorted(set().union(*[e.free_symbols for e in exprs]), key=lambda s: s.name)
    names = {s: f"s{k}" for k, s in enumerate(syms)}
    fold = _folds_inv_dd(low, fast)
    if fold:
        laps = [s for s in syms if _parse(s)[0] == "y-laplacian"]
        exprs = [e.subs({s: s * INV_DD for s in laps}) for e in exprs]
        names[INV_DD] = "a.inv_dd()"
    printer = _KernelPrinter(names, fast)
    lines = [
        f"  template <class P> static __device__ __forceinline__ void {name}"
        f"(const P& a, typename P::real* f{tail}) {{",
        "    using T = typename P::real;",
    ]
    for s in syms:
        code = _symbol_code(s, low, fast)
        if fold and _parse(s)[0] == "y-laplacian":
            code = f"a.template lapr<{_parse(s)[1][0]}>()"
        lines.append(f"    const T {names[s]} = {code};  // {s.name}")
    for k, e in enumerate(exprs):
        parts = _const_split(e) if split else None
        if split and parts is None:
            parts = (sp.Integer(1), e)
        if split:
            lines.append(f"    f[{k}] = {printer.doprint(parts[1])};")
            lines.append(f"    fk[{k}] = {printer.doprint(parts[0])};")
        else:
            lines.append(f"    f[{k}] = {printer.doprint(e)};")
    lines.append("  }")
    return "\n".join(lines) + "\n"


_TEMPLATE_FILES = (
    ("csrc", "fdm_step.cuh"),
    ("csrc", "fdm_step3d.cuh"),
    ("include", "prml_params.h"),
)


def _template_digest() -> str:
    """Hash of the headers every generated module includes (part of the cubin cache key)."""
    import os

    pkg = os.path.dirname(os.path.abspath(__file__))
    roots = {"csrc": os.path.join(pkg, "csrc"), "include": os.path.join(os.path.dirname(pkg), "include")}
    h = hashlib.sha256()
    for root, name in _TEMPLATE_FILES:
        with open(os.path.join(roots[root], name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _chain(values: Sequence[int]) -> str:
    expr = "-1"
    for k in reversed(range(len(values))):
        expr = f"(i == {k} ? {values[k]} : {expr})"
    return expr


def tile_steps(tile) -> int:
    """Time steps one launch of a tile's kernel takes (4th entry, default 1)."""
    return int(tile[3]) if len(tile) > 3 else 1


def tile_planes(tile) -> int:
    """Tile depth (planes) of a 3D kernel's tile (5th entry), 0 for 2D tiles."""
    return int(tile[4]) if len(tile) > 4 else 0


def is_walk(tile) -> bool:
    """Whether a tile key names a register-window kernel (walk_body)."""
    return len(tile) > 5 and tile[5] == "w"


def walk_tile(rows_per_thread: int, warps: int, esize: int) -> tuple:
    """Tile key of the register-window kernel with R rows per thread and
    ``warps`` warps per CTA."""
    return (4 * rows_per_thread, warps * 8 * (16 // esize), 32 * warps, 1, 0, "w")


def kernel_name(kind: str, dtype: str, tile) -> str:
    if is_walk(tile):
        return f"prml_walk_{dtype}_{tile[0]}x{tile[1]}x{tile[2]}"
    if tile_planes(tile):
        return f"prml_{kind}_{dtype}_{tile_planes(tile)}x{tile[0]}x{tile[1]}x{tile[2]}"
    name = f"prml_{kind}_{dtype}_{tile[0]}x{tile[1]}x{tile[2]}"
    return name if tile_steps(tile) == 1 else f"{name}_k{tile_steps(tile)}"


def stage_count(integrator: int, invariant: bool, mode: int) -> int:
    return 1 if (mode == 1 or invariant) else integrator


def halo(integrator: int, invariant: bool, mode: int, tile) -> int:
    """Row halo of a kernel's staged region: its stage count, or the number
    of steps of a temporally blocked kernel."""
    k = tile_steps(tile)
    return k if k > 1 else stage_count(integrator, invariant, mode)


def col_halo(nstage: int, esize: int) -> int:
    """Column halo: >= the stage count, rounded up to 16 bytes (TMA alignment)."""
    align = 16 // esize
    return (nstage + align - 1) // align * align


def region(tile, nstage: int, esize: int) -> Tuple[int, int]:
    """(rows, cols) of the staged tile + halo; also the TMA box extents."""
    return tile[0] + 2 * nstage, tile[1] + 2 * col_halo(nstage, esize)


def buffer_count(integrator: int, invariant: bool, mode: int, tile) -> int:
    """Shared buffers of a kernel: two TMA staging buffers plus the on-chip
    stage (or step) inputs."""
    k = tile_steps(tile)
    if k > 1:
        return 2 + (1 if k == 2 else 2)
    nstage = stage_count(integrator, invariant, mode)
    return 2 + (0 if nstage == 1 else (1 if nstage == 2 else 2))


def staged_planes(n_comp: int, comp: bool, tile) -> int:
    """Planes per staged region: a blocked compensated state carries its lo planes."""
    return 2 * n_comp if (comp and tile_steps(tile) > 1) else n_comp


def smem_bytes(low: LoweredProblem, integrator: int, invariant: bool, tile, esize: int, mode: int,
               comp: bool = False) -> int:
    h = halo(integrator, invariant, mode, tile)
    rx, ry = region(tile, h, esize)
    planes = staged_planes(low.n_comp, comp, tile)
    depth = tile_planes(tile) + 2 * h if tile_planes(tile) else 1
    buf = (planes * depth * rx * ry * esize + 127) // 128 * 128  # 128-byte aligned buffers
    return buffer_count(integrator, invariant, mode, tile) * buf + 128 + 16  # + base alignment slack + two mbarriers


@dataclasses.dataclass
class GeneratedModule:
    source: str
    key: str
    dtype: str
    integrator: int
    invariant: bool
    step_kernels: Dict[tuple, Tuple[str, int]]  # tile (rows, cols, threads[, steps]) -> (name, smem)
    rhs_kernel: Tuple[str, int, Tuple[int, int, int]]
    n_comp: int = 1
    multi_kernels: Dict[tuple, Tuple[str, int]] = dataclasses.field(default_factory=dict)

    def box(self, tile, mode: int = 0) -> Tuple[int, int]:
        """TMA box (rows, cols) a kernel of this module stages."""
        esize = 8 if self.dtype == "f64" else 4
        return region(tile, halo(self.integrator, self.invariant, mode, tile), esize)

    def box_planes(self, tile) -> int:
        """Component planes of the TMA box of a step kernel."""
        return staged_planes(self.n_comp, self.dtype == "f32c", tile)

    def box_depth(self, tile, mode: int = 0) -> int:
        """Mesh planes of the TMA box of a 3D kernel (1 for 2D kernels)."""
        if not tile_planes(tile):
            return 1
        return tile_planes(tile) + 2 * halo(self.integrator, self.invariant, mode, tile)


def generate_source(low: LoweredProblem, integrator: int, dtype: str, exact_div: bool = False,
                    fast: bool = False, multi: bool = False) -> GeneratedModule:
    """CUDA source of one module: the equation struct plus step kernels.

    ``exact_div``: the Cartesian differences divide by 2 dx and dx^2 as the
    reference's numpy expressions do (float64 right-hand sides of the
    implicit integrators, whose secant stop test turns one-ulp differences
    into differences of the order of its tolerance) instead of multiplying
    by reciprocals.

    ``fast`` (fused operation order; 1D and 2D meshes, not with
    ``exact_div``): the Cartesian Laplacian is one neighbour sum minus four
    (two per axis) times the centre, scaled once; sums with a product term
    are multiply-adds; the integrator combines unscaled slopes and scales
    them once (a stage-invariant RK4 step is y + dt f).  Each result stays
    within a few roundings of the reference's operation order, with about
    half the floating-point operations per vertex (the float64 pipe of this
    GPU issues about two operations per clock per SM).

    ``multi``: also instantiate the multi-round kernels (``multi_body``: every
    step of several groups of instances in one cooperative launch)."""
    if integrator not in (FORWARD_EULER, EXPLICIT_MIDPOINT, RK4):
        raise ValueError(f"unsupported integrator {integrator}")
    fast = bool(fast) and not exact_div and low.x_dimension != 3
    ctype = {"f32": "float", "f32c": "float", "f64": "double"}[dtype]
    esize = 8 if dtype == "f64" else 4
    comp = 1 if dtype == "f32c" else 0
    invariant = is_stage_invariant(low, integrator)
    # whether any right-hand side reads t (else the kernels skip time arithmetic)
    uses_t = any(sym.name == "t" for expr in low.rhs for sym in expr.free_symbols)
    d_rows, y_rows = list(low.d_idx), list(low.y_idx)
    three_d = low.x_dimension == 3
    if three_d and comp:
        raise NotImplementedError("compensated float32 is not available on 3D meshes")
    body = [
        '#include "fdm_step3d.cuh"' if three_d else '#include "fdm_step.cuh"',
        "",
        "struct Eq {",
        f"  static constexpr int C = {low.n_comp};",
        f"  static constexpr int ND = {len(d_rows)};",
        f"  static constexpr int NYC = {len(y_rows)};",
        f"  static constexpr bool STAGE_INVARIANT = {'true' if invariant else 'false'};",
        f"  static constexpr bool USES_T = {'true' if uses_t else 'false'};",
        f"  static constexpr bool EXACT_DIV = {'true' if exact_div else 'false'};",
        f"  static constexpr bool FAST = {'true' if fast else 'false'};",
        f"  static constexpr bool EQUAL_DX = {'true' if low.dx_k[0] == low.dx_k[1] else 'false'};",
        f"  static constexpr unsigned long long NEU_MASK = {low.neu_mask}ull;",
        f"  static constexpr unsigned long long DIR_MASK = {low.dir_mask}ull;",
        f"  static __device__ constexpr int dcomp(int i) {{ return {_chain(d_rows)}; }}",
        f"  static __device__ constexpr int ycomp(int i) {{ return {_chain(y_rows)}; }}",
        _rhs_function("rhs_dt", d_rows, low, fast),
        _rhs_function("rhs_y", y_rows, low, fast),
        _rhs_function("rhs_dt_split", d_rows, low, fast, split=True) if fast else "",
        "};",
        "",
    ]
    step_kernels = {}
    single_stage = stage_count(integrator, invariant, 0) == 1
    if three_d:
        for tile in TILE_CONFIGS_3D:
            sm = smem_bytes(low, integrator, invariant, tile, esize, 0)
            if sm > SMEM_LIMIT:
                continue
            name = kernel_name("step", dtype, tile)
            step_kernels[tile] = (name, sm)
            body.append(
                f'extern "C" __global__ void __launch_bounds__({tile[2]}) {name}'
                f"(const prml_step_params p, const __grid_constant__ prml::TmaDesc tin) "
                f"{{ prml::step_body3<{ctype}, Eq, {integrator}, {tile_planes(tile)}, {tile[0]}, {tile[1]}, "
                f"{tile[2]}, 0>(p, tin); }}"
            )
        if not step_kernels:
            raise NotImplementedError("no 3D tile configuration fits in shared memory")
        rtile = (4, 32, 128, 1, 2)
        rname = kernel_name("rhs", dtype, rtile)
        rsm = smem_bytes(low, integrator, invariant, rtile, esize, 1)
        body.append(
            f'extern "C" __global__ void __launch_bounds__({rtile[2]}) {rname}'
            f"(const prml_step_params p, const __grid_constant__ prml::TmaDesc tin) "
            f"{{ prml::step_body3<{ctype}, Eq, {integrator}, {rtile[4]}, {rtile[0]}, {rtile[1]}, {rtile[2]}, 1>(p, tin); }}"
        )
        source = "\n".join(body) + "\n"
        key = hashlib.sha256((source + _template_digest()).encode()).hexdigest()[:24]
        return GeneratedModule(source=source, key=key, dtype=dtype, integrator=integrator, invariant=invariant,
                               step_kernels=step_kernels, rhs_kernel=(rname, rsm, rtile), n_comp=low.n_comp)
    # temporally blocked kernels take several steps per launch; a Jacobi
    # solve has to run between every two steps
    blocked = single_stage and not low.lap_idx
    for tile in TILE_CONFIGS + (TB_CONFIGS if blocked else ()):
        sm = smem_bytes(low, integrator, invariant, tile, esize, 0, comp=bool(comp))
        if sm > SMEM_LIMIT:
            continue
        name = kernel_name("step", dtype, tile)
        step_kernels[tile] = (name, sm)
        # one single-stage step per launch: cap registers at 32 so a full SM
        # of CTAs (2048 threads) stays resident and one round covers the mesh
        minb = f", {2048 // tile[2]}" if (single_stage and tile_steps(tile) == 1) else ""
        body.append(
            f'extern "C" __global__ void __launch_bounds__({tile[2]}{minb}) {name}'
            f"(const prml_step_params p, const __grid_constant__ prml::TmaDesc tin) "
            f"{{ prml::step_body<{ctype}, Eq, {integrator}, {tile[0]}, {tile[1]}, {tile[2]}, 0, {comp}, "
            f"{tile_steps(tile)}>(p, tin); }}"
        )
    if single_stage and low.x_dimension == 2:
        # register-window kernels: no staging, the window in registers
        for r_rows, warps in WALK_CONFIGS:
            tile = walk_tile(r_rows, warps, esize)
            name = kernel_name("step", dtype, tile)
            step_kernels[tile] = (name, 0)
            body.append(
                f'extern "C" __global__ void __launch_bounds__({tile[2]}) {name}'
                f"(const prml_step_params p, const __grid_constant__ prml::TmaDesc tin) "
                f"{{ (void)tin; prml::walk_body<{ctype}, Eq, {integrator}, {r_rows}, {warps}, {comp}>(p); }}"
            )
    if not step_kernels:
        raise NotImplementedError("no tile configuration fits in shared memory")
    rtile = (16, 32, 128)
    rname = kernel_name("rhs", dtype, rtile)
    rsm = smem_bytes(low, integrator, invariant, rtile, esize, 1)
    body.append(
        f'extern "C" __global__ void __launch_bounds__({rtile[2]}) {rname}'
        f"(const prml_step_params p, const __grid_constant__ prml::TmaDesc tin) "
        f"{{ prml::step_body<{ctype}, Eq, {integrator}, {rtile[0]}, {rtile[1]}, {rtile[2]}, 1>(p, tin); }}"
    )
    # multi-round kernels: every step of several groups in one cooperative
    # launch (not for Jacobi rows, which need a solve between two steps)
    multi_kernels = {}
    if multi and not low.lap_idx:
        for tile in MULTI_TILES:
            sm = smem_bytes(low, integrator, invariant, tile, esize, 0)
            if sm + MULTI_STATIC_SMEM > SMEM_LIMIT:
                continue
            name = kernel_name("multi", dtype, tile)
            multi_kernels[tile] = (name, sm)
            body.append(
                f'extern "C" __global__ void __launch_bounds__({tile[2]}) {name}(const prml_multi_params mp) '
                f"{{ prml::multi_body<{ctype}, Eq, {integrator}, {tile[0]}, {tile[1]}, {tile[2]}, {comp}>(mp); }}"
            )
    source = "\n".join(body) + "\n"
    key = hashlib.sha256((source + _template_digest()).encode()).hexdigest()[:24]
    return GeneratedModule(
        source=source,
        key=key,
        dtype=dtype,
        integrator=integrator,
        invariant=invariant,
        step_kernels=step_kernels,
        rhs_kernel=(rname, rsm, rtile),
        n_comp=low.n_comp,
        multi_kernels=multi_kernels,
    )
