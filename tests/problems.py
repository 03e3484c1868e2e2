"""Problem builders shared by the tests, the fixture generator and the bench.

Each builder takes a namespace ``ns`` exposing PararealML's public classes —
either this package (``pararealml_gb300``) or the reference package itself —
and returns an initial value problem, so the same definition runs through the
reference (to make golden fixtures) and through the GPU path.
"""

from __future__ import annotations

import numpy as np

SEEDS = [541016860, 890237211, 110287329, 734589112]


def zeros_bc(n_comp):
    return lambda x, t: np.zeros((len(x), n_comp))


def diffusion_2d(ns, n=64, t_end=2.0):
    """2D diffusion, [0,10]^2, zero Dirichlet, Gaussian peak 1 at (5, 5)."""
    diff_eq = ns.DiffusionEquation(2, 1.0)
    mesh = ns.Mesh([(0.0, 10.0), (0.0, 10.0)], [10.0 / n, 10.0 / n])
    bc = ns.DirichletBoundaryCondition(zeros_bc(1), is_static=True)
    cp = ns.ConstrainedProblem(diff_eq, mesh, [(bc, bc)] * 2)
    ic = ns.GaussianInitialCondition(cp, [(np.array([5.0, 5.0]), 0.5 * np.eye(2))], [np.pi])
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def cahn_hilliard_2d(ns, n=32, length=8.0, t_end=0.05, seed=SEEDS[0], gamma=0.01, d=0.1):
    """Cahn-Hilliard on [0,L]^2, zero-flux Neumann, c0 ~ U(-0.1, 0.1),
    mu0 = c0^3 - c0 - gamma lap(c0) with the Neumann derivative constraints."""
    diff_eq = ns.CahnHilliardEquation(2, d, gamma)
    mesh = ns.Mesh([(0.0, length), (0.0, length)], [length / n, length / n])
    bc = ns.NeumannBoundaryCondition(zeros_bc(2), is_static=True)
    cp = ns.ConstrainedProblem(diff_eq, mesh, [(bc, bc)] * 2)
    rng = np.random.default_rng(seed)
    c0 = rng.uniform(-0.1, 0.1, mesh.vertices_shape + (1,))
    mu0 = c0**3 - c0 - gamma * _neumann_laplacian(c0, mesh.d_x)
    ic = ns.DiscreteInitialCondition(cp, np.concatenate([c0, mu0], axis=-1), True)
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def _neumann_laplacian(y, d_x):
    """Laplacian of one component with zero Neumann ghosts (y[1], y[n-2])."""
    out = np.zeros_like(y)
    for axis in range(y.ndim - 1):
        sl = [slice(None)] * y.ndim
        sl[axis] = slice(1, 2)
        lo = y[tuple(sl)]
        sl[axis] = slice(-2, -1)
        hi = y[tuple(sl)]
        ext = np.concatenate([lo, y, hi], axis=axis)
        a = [slice(None)] * y.ndim
        b = [slice(None)] * y.ndim
        c = [slice(None)] * y.ndim
        a[axis], b[axis], c[axis] = slice(0, -2), slice(1, -1), slice(2, None)
        out += (ext[tuple(c)] - 2.0 * ext[tuple(b)] + ext[tuple(a)]) / (d_x[axis] * d_x[axis])
    return out


def shallow_water_2d(ns, n=32, length=64.0, t_end=0.5, amp=0.1, centre=(30.0, 34.0), g=9.81):
    """Shallow water (h, u, v); zero-flux on h only (u, v free), Gaussian bump."""
    diff_eq = ns.ShallowWaterEquation(1.0, g=g)
    mesh = ns.Mesh([(0.0, length), (0.0, length)], [length / n, length / n])
    bc = ns.NeumannBoundaryCondition(
        ns.vectorize_bc_function(lambda x, t: (0.0, None, None)), is_static=True
    )
    cp = ns.ConstrainedProblem(diff_eq, mesh, [(bc, bc)] * 2)
    var = 0.25 * (length / 8.0) ** 2
    ic = ns.GaussianInitialCondition(
        cp, [(np.array(centre), var * np.eye(2))] * 3, [amp * 2 * np.pi * var, 0.0, 0.0]
    )
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def mixed_bc_wave_2d(ns, nx=24, ny=20, t_end=0.1):
    """Wave equation with non-zero, partially masked Dirichlet values, a
    Neumann face and a free face: exercises corner precedence and NaN masks."""
    diff_eq = ns.WaveEquation(2, 0.7)
    mesh = ns.Mesh([(-1.0, 2.0), (0.0, 2.5)], [3.0 / nx, 2.5 / ny])

    def lower0(x, t):
        v = np.stack([np.sin(x[:, 1]), np.full(len(x), np.nan)], axis=-1)
        return v

    def upper0(x, t):
        return np.stack([0.5 + 0.1 * x[:, 1], np.cos(x[:, 1])], axis=-1)

    def lower1(x, t):
        v = np.stack([x[:, 0] * 0.3, np.full(len(x), np.nan)], axis=-1)
        v[x[:, 0] > 1.0, 0] = np.nan
        return v

    bcs = [
        (
            ns.DirichletBoundaryCondition(lower0, is_static=True),
            ns.DirichletBoundaryCondition(upper0, is_static=True),
        ),
        (
            ns.NeumannBoundaryCondition(lower1, is_static=True),
            ns.NeumannBoundaryCondition(lambda x, t: np.full((len(x), 2), 0.25), is_static=True),
        ),
    ]
    cp = ns.ConstrainedProblem(diff_eq, mesh, bcs)
    ic = ns.GaussianInitialCondition(
        cp, [(np.array([0.5, 1.2]), 0.2 * np.eye(2)), (np.array([0.4, 1.0]), 0.3 * np.eye(2))], [1.0, 0.5]
    )
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def burgers_2d(ns, n=24, t_end=0.05, re=50.0):
    """Burgers (gradient-heavy nonlinear RHS) with mixed Cauchy/Dirichlet BCs."""
    diff_eq = ns.BurgersEquation(2, re)
    mesh = ns.Mesh([(0.0, 1.0), (0.0, 1.0)], [1.0 / n, 1.0 / n])
    bc_d = ns.DirichletBoundaryCondition(lambda x, t: np.zeros((len(x), 2)), is_static=True)
    bc_c = ns.CauchyBoundaryCondition(
        lambda x, t: np.stack([0.1 * np.ones(len(x)), np.full(len(x), np.nan)], -1),
        lambda x, t: np.stack([np.full(len(x), np.nan), -0.2 * np.ones(len(x))], -1),
        is_static=True,
    )
    cp = ns.ConstrainedProblem(diff_eq, mesh, [(bc_d, bc_c), (bc_c, bc_d)])
    ic = ns.GaussianInitialCondition(
        cp, [(np.array([0.5, 0.5]), 0.02 * np.eye(2)), (np.array([0.4, 0.6]), 0.03 * np.eye(2))], [0.3, -0.2]
    )
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def convection_diffusion_1d(ns, n=50, t_end=0.2):
    """1D convection-diffusion with a Neumann lower and Dirichlet upper end."""
    diff_eq = ns.ConvectionDiffusionEquation(1, [0.8], 0.05)
    mesh = ns.Mesh([(0.0, 5.0)], [5.0 / n])
    bcs = [
        (
            ns.NeumannBoundaryCondition(lambda x, t: np.full((len(x), 1), 0.3), is_static=True),
            ns.DirichletBoundaryCondition(lambda x, t: np.full((len(x), 1), 0.1), is_static=True),
        )
    ]
    cp = ns.ConstrainedProblem(diff_eq, mesh, bcs)
    ic = ns.GaussianInitialCondition(cp, [(np.array([2.0]), np.array([[0.3]]))], [1.0])
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def population_growth(ns, t_end=1.0):
    """ODE (no mesh): dy/dt = r y."""
    diff_eq = ns.PopulationGrowthEquation(0.5)
    cp = ns.ConstrainedProblem(diff_eq)
    ic = ns.ConstantInitialCondition(cp, [100.0])
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def shallow_water_ensemble(ns, n_instances=256, sizes=(64, 128, 256, 512), length=64.0, t_end=1.0,
                           seed=SEEDS[3], g=9.81, cfl=0.4):
    """Shallow water (h, u, v) instances on meshes of mixed size,
    zero-flux on h (u, v free), Gaussian bumps of amplitude U(0.05, 0.2) at
    centres U([8, 56]^2) with covariance 0.25 I, u = v = 0, RK4 at CFL
    ``cfl`` per mesh (dt = t_end / ceil(t_end / (cfl dx / sqrt(g h0))))."""
    rng = np.random.default_rng(seed)
    eq = ns.ShallowWaterEquation(1.0, g=g)
    bc = ns.NeumannBoundaryCondition(ns.vectorize_bc_function(lambda x, t: (0.0, None, None)), is_static=True)
    cps = {n: ns.ConstrainedProblem(eq, ns.Mesh([(0.0, length)] * 2, [length / n] * 2), [(bc, bc)] * 2) for n in sizes}
    ivps, d_ts = [], []
    for _ in range(n_instances):
        n = sizes[int(rng.integers(len(sizes)))]
        amp = rng.uniform(0.05, 0.2)
        centre = rng.uniform(8.0, length - 8.0, 2)
        cp = cps[n]
        ic = ns.GaussianInitialCondition(cp, [(centre, 0.25 * np.eye(2))] * 3, [amp * 2 * np.pi * 0.25, 0.0, 0.0])
        ivps.append(ns.InitialValueProblem(cp, (0.0, t_end), ic))
        dt_max = cfl * (length / n) / np.sqrt(g * 1.0)
        steps = int(np.ceil(t_end / dt_max))
        d_ts.append(t_end / steps)
    return ivps, d_ts


def dynamic_bc_diffusion_1d(ns):
    """The reference's own time-dependent boundary test problem
    (tests/operators/fdm/test_fdm_operator.py:293-319): 1D diffusion, zero
    Neumann lower end, Dirichlet upper end rising as t / 5 (both dynamic)."""
    diff_eq = ns.DiffusionEquation(1, 1.5)
    mesh = ns.Mesh([(0.0, 10.0)], [1.0])
    bcs = [
        (
            ns.NeumannBoundaryCondition(lambda x, t: np.zeros((len(x), 1))),
            ns.DirichletBoundaryCondition(lambda x, t: np.full((len(x), 1), t / 5.0)),
        )
    ]
    cp = ns.ConstrainedProblem(diff_eq, mesh, bcs)
    ic = ns.GaussianInitialCondition(cp, [(np.array([5.0]), np.array([[2.5]]))], [20.0])
    return ns.InitialValueProblem(cp, (0.0, 10.0), ic)


def dynamic_bc_wave_2d(ns, nx=26, ny=21, t_end=0.04):
    """Wave equation (y, dy/dt) with time-dependent Dirichlet and Neumann
    faces whose values vary along the face and are NaN-masked in part, and
    a start time away from zero."""
    diff_eq = ns.WaveEquation(2, 0.7)
    mesh = ns.Mesh([(-1.0, 2.0), (0.0, 2.5)], [3.0 / nx, 2.5 / ny])

    def lower0(x, t):
        return np.stack([np.sin(x[:, 1] + 3.0 * t), np.full(len(x), np.nan)], axis=-1)

    def upper0(x, t):
        return np.stack([0.2 * np.cos(2.0 * t) + 0.1 * x[:, 1], np.full(len(x), 0.05 * t)], axis=-1)

    def lower1(x, t):
        v = np.stack([0.5 * t * x[:, 0], np.full(len(x), np.nan)], axis=-1)
        v[x[:, 0] > 1.0, 0] = np.nan
        return v

    def upper1(x, t):
        return np.full((len(x), 2), 0.25 + t)

    bcs = [
        (ns.DirichletBoundaryCondition(lower0), ns.NeumannBoundaryCondition(upper0)),
        (ns.DirichletBoundaryCondition(lower1), ns.NeumannBoundaryCondition(upper1)),
    ]
    cp = ns.ConstrainedProblem(diff_eq, mesh, bcs)
    ic = ns.GaussianInitialCondition(
        cp, [(np.array([0.5, 1.2]), 0.2 * np.eye(2)), (np.array([0.4, 1.0]), 0.3 * np.eye(2))], [1.0, 0.5]
    )
    return ns.InitialValueProblem(cp, (0.3, 0.3 + t_end), ic)


def cahn_hilliard_3d(ns, t_end=0.5, seed=SEEDS[1]):
    """The reference's own 3D test problem (tests/operators/fdm/
    test_fdm_operator.py:173-197): Cahn-Hilliard on [0,5] x [0,5] x [0,10]
    with steps 0.5, 1, 2 (11 x 6 x 6 vertices), zero-flux Neumann, both
    components 0.05 U(-1, 1) (seeded here)."""
    diff_eq = ns.CahnHilliardEquation(3)
    mesh = ns.Mesh([(0.0, 5.0), (0.0, 5.0), (0.0, 10.0)], [0.5, 1.0, 2.0])
    bc = ns.NeumannBoundaryCondition(zeros_bc(2), is_static=True)
    cp = ns.ConstrainedProblem(diff_eq, mesh, [(bc, bc)] * 3)
    rng = np.random.default_rng(seed)
    ic = ns.DiscreteInitialCondition(cp, 0.05 * rng.uniform(-1.0, 1.0, cp.y_shape(True)), True)
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def diffusion_3d_mixed(ns, n=(9, 12, 14), t_end=0.02):
    """3D diffusion with Dirichlet values varying along two faces (NaN-masked
    in part), Neumann faces and a free face pair; Gaussian bump."""
    diff_eq = ns.DiffusionEquation(3, 0.8)
    mesh = ns.Mesh([(0.0, 2.0), (0.0, 3.0), (-1.0, 2.5)], [2.0 / n[0], 3.0 / n[1], 3.5 / n[2]])

    def dir_lo(x, t):
        v = (0.1 * x[:, 1] + 0.05 * x[:, 2])[:, None]
        v[x[:, 1] > 2.0] = np.nan
        return v

    bcs = [
        (ns.DirichletBoundaryCondition(dir_lo, is_static=True),
         ns.NeumannBoundaryCondition(lambda x, t: np.full((len(x), 1), 0.3), is_static=True)),
        (ns.NeumannBoundaryCondition(lambda x, t: (0.2 * x[:, 0])[:, None], is_static=True),
         ns.DirichletBoundaryCondition(lambda x, t: np.full((len(x), 1), 0.5), is_static=True)),
        (ns.NeumannBoundaryCondition(zeros_bc(1), is_static=True),
         ns.NeumannBoundaryCondition(zeros_bc(1), is_static=True)),
    ]
    cp = ns.ConstrainedProblem(diff_eq, mesh, bcs)
    ic = ns.GaussianInitialCondition(cp, [(np.array([1.0, 1.5, 0.5]), 0.3 * np.eye(3))], [2.0])
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def polar_shallow_water(ns, t_end=1.0):
    """The reference's polar test problem (tests/operators/fdm/
    test_fdm_operator.py:200-232): shallow water on an annulus."""
    diff_eq = ns.ShallowWaterEquation(0.5)
    mesh = ns.Mesh([(1.0, 11.0), (0.0, 2 * np.pi)], [2.0, np.pi / 5.0], ns.CoordinateSystem.POLAR)
    bc = ns.NeumannBoundaryCondition(ns.vectorize_bc_function(lambda x, t: (0.0, None, None)), is_static=True)
    cp = ns.ConstrainedProblem(diff_eq, mesh, [(bc, bc)] * 2)
    ic = ns.GaussianInitialCondition(
        cp, [(np.array([-6.0, 0.0]), np.array([[0.25, 0.0], [0.0, 0.25]]))] * 3, [1.0, 0.0, 0.0]
    )
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def curvilinear_diffusion_3d(ns, system: str = "CYLINDRICAL", t_end=1.0):
    """The reference's cylindrical and spherical test problems
    (tests/operators/fdm/test_fdm_operator.py:235-290): diffusion with
    zero-flux faces from y0 = 1 / r."""
    cs = getattr(ns.CoordinateSystem, system)
    if system == "CYLINDRICAL":
        mesh = ns.Mesh([(1.0, 11.0), (0.0, 2 * np.pi), (0.0, 2.0)], [2.0, np.pi / 5.0, 1.0], cs)
    else:
        mesh = ns.Mesh([(1.0, 11.0), (0.0, 2.0 * np.pi), (0.1 * np.pi, 0.9 * np.pi)],
                       [2.0, np.pi / 5.0, np.pi / 5], cs)
    bc = ns.NeumannBoundaryCondition(zeros_bc(1), is_static=True)
    cp = ns.ConstrainedProblem(ns.DiffusionEquation(3), mesh, [(bc, bc)] * 3)
    ic = ns.ContinuousInitialCondition(cp, lambda x: 1.0 / x[:, :1])
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def curvilinear_vector_field(ns, system: str = "SPHERICAL", t_end=0.01):
    """A 3-component field on a spherical / cylindrical mesh whose right-hand
    sides use every curvilinear operator: gradients, Hessians (mixed and
    pure), Laplacian, divergence and the three curl components; Neumann
    values on some faces."""
    import sympy as sp

    class VectorField(ns.DifferentialEquation):
        def __init__(self):
            super().__init__(3, 3)

        @property
        def symbolic_equation_system(self):
            s = self.symbols
            y, g, h, lap = s.y, s.y_gradient, s.y_hessian, s.y_laplacian
            div = s.y_divergence[0, 1, 2]
            curl = s.y_curl[0, 1, 2]
            return ns.SymbolicEquationSystem([
                0.05 * lap[0] + 0.01 * h[0, 0, 1] - 0.02 * g[1, 2] + 0.03 * curl[0],
                0.04 * lap[1] + 0.01 * h[1, 1, 2] + 0.02 * div + 0.01 * curl[1] - 0.1 * y[1],
                0.03 * h[2, 2, 2] + 0.02 * h[2, 1, 1] + 0.01 * h[2, 0, 2] + 0.02 * curl[2] + 0.05 * g[0, 0],
            ])

    cs = getattr(ns.CoordinateSystem, system)
    if system == "SPHERICAL":
        mesh = ns.Mesh([(1.0, 3.0), (0.0, np.pi), (0.2 * np.pi, 0.8 * np.pi)], [0.25, np.pi / 8, np.pi / 10], cs)
    else:
        mesh = ns.Mesh([(1.0, 3.0), (0.0, np.pi), (0.0, 2.0)], [0.25, np.pi / 8, 0.25], cs)
    neu = ns.NeumannBoundaryCondition(lambda x, t: np.stack([0.1 * x[:, 0], np.zeros(len(x)), np.full(len(x), np.nan)], -1),
                                      is_static=True)
    free = ns.NeumannBoundaryCondition(lambda x, t: np.full((len(x), 3), np.nan), is_static=True)
    cp = ns.ConstrainedProblem(VectorField(), mesh, [(neu, free), (free, neu), (neu, neu)])
    ic = ns.ContinuousInitialCondition(
        cp, lambda x: np.stack([np.sin(x[:, 1]) / x[:, 0], np.cos(x[:, 2]) * x[:, 0], 0.1 * x[:, 0] ** 2], -1)
    )
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


# seed of numpy's global generator before a solve with LHS.Y_LAPLACIAN rows:
# every step's Jacobi solve starts from np.random.random (the reference's
# numerical_differentiator.py:910-911), drawn in the same order by the GPU path
JACOBI_SEED = 20240617


def navier_stokes_2d(ns, n=10, length=10.0, t_end=10.0, re=5000.0):
    """The reference's own 2D test problem (tests/operators/fdm/
    test_fdm_operator.py:136-170): vorticity / stream function / velocity on
    an 11 x 11 mesh, Dirichlet vorticity and stream function on every face,
    from rest; the stream function is the LHS.Y_LAPLACIAN row."""
    diff_eq = ns.NavierStokesEquation(re)
    mesh = ns.Mesh([(0.0, length), (0.0, length)], [length / n, length / n])
    vec = ns.vectorize_bc_function
    bcs = [
        (ns.DirichletBoundaryCondition(vec(lambda x, t: (1.0, 0.1, None, None)), is_static=True),
         ns.DirichletBoundaryCondition(vec(lambda x, t: (0.0, 0.0, None, None)), is_static=True)),
        (ns.DirichletBoundaryCondition(vec(lambda x, t: (0.0, 0.0, None, None)), is_static=True),
         ns.DirichletBoundaryCondition(vec(lambda x, t: (0.0, 0.0, None, None)), is_static=True)),
    ]
    cp = ns.ConstrainedProblem(diff_eq, mesh, bcs)
    ic = ns.ContinuousInitialCondition(cp, lambda x: np.zeros((len(x), 4)))
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


_JACOBI_MESHES = {
    ("CARTESIAN", 1): ([(0.0, 2.0)], [0.1]),
    ("CARTESIAN", 2): ([(0.0, 2.0), (-1.0, 1.5)], [2.0 / 14, 2.5 / 11]),
    ("CARTESIAN", 3): ([(0.0, 1.0), (0.0, 1.2), (0.0, 1.4)], [1.0 / 7, 1.2 / 8, 1.4 / 9]),
    ("POLAR", 2): ([(1.0, 3.0), (0.0, np.pi)], [0.2, np.pi / 10]),
    ("CYLINDRICAL", 3): ([(1.0, 3.0), (0.0, np.pi), (0.0, 1.0)], [0.25, np.pi / 8, 0.2]),
    ("SPHERICAL", 3): ([(1.0, 3.0), (0.0, np.pi), (0.2 * np.pi, 0.8 * np.pi)], [0.25, np.pi / 8, np.pi / 10]),
}


def jacobi_system(ns, system="CARTESIAN", dims=2, t_end=0.02, dynamic=False, mesh=None):
    """A two-component system with an LHS.Y_LAPLACIAN row on any mesh:
    du/dt = 0.1 lap(u) + 0.5 psi and lap(psi) = u - 0.3 x0.  Every axis has
    a Dirichlet face and a Neumann face (non-zero values, the stream
    function's Neumann values NaN-masked on part of one face), so the Jacobi
    solve meets Dirichlet values, Neumann ghosts and zero halos;
    ``dynamic``: the first face's values change with t; ``mesh``: (bounds,
    steps) instead of the small mesh of the coordinate system."""
    class Coupled(ns.DifferentialEquation):
        def __init__(self):
            super().__init__(dims, 2)

        @property
        def symbolic_equation_system(self):
            s = self.symbols
            return ns.SymbolicEquationSystem(
                [0.1 * s.y_laplacian[0] + 0.5 * s.y[1], s.y[0] - 0.3 * s.x[0]],
                [ns.LHS.D_Y_OVER_D_T, ns.LHS.Y_LAPLACIAN],
            )

    bounds, steps = mesh if mesh is not None else _JACOBI_MESHES[(system, dims)]
    mesh = ns.Mesh(bounds, steps, getattr(ns.CoordinateSystem, system))

    def dir_lo(x, t):
        return np.stack([0.2 + 0.1 * x[:, -1] + (t if dynamic else 0.0), np.full(len(x), 0.05)], -1)

    def neu_hi(x, t):
        v = np.stack([np.full(len(x), -0.1), 0.2 * np.ones(len(x))], -1)
        v[x[:, 0] > 0.5 * (bounds[0][0] + bounds[0][1]), 1] = np.nan
        return v

    def neu_lo(x, t):
        return np.stack([np.zeros(len(x)), np.full(len(x), 0.1)], -1)

    def dir_hi(x, t):
        return np.stack([np.full(len(x), 0.3), -0.05 * x[:, 0]], -1)

    pairs = []
    for axis in range(dims):
        if axis % 2 == 0:
            pairs.append((ns.DirichletBoundaryCondition(dir_lo, is_static=not (dynamic and axis == 0)),
                          ns.NeumannBoundaryCondition(neu_hi, is_static=True)))
        else:
            pairs.append((ns.NeumannBoundaryCondition(neu_lo, is_static=True),
                          ns.DirichletBoundaryCondition(dir_hi, is_static=True)))
    cp = ns.ConstrainedProblem(Coupled(), mesh, pairs)
    ic = ns.ContinuousInitialCondition(
        cp, lambda x: np.stack([0.3 + 0.2 * np.sin(x[:, 0]) * np.cos(x[:, -1]), np.zeros(len(x))], -1))
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)


def navier_stokes_example(ns, n_steps=10, d_t=0.05):
    """The reference's Navier-Stokes example (examples/navier_stokes_fdm.py):
    Re = 5000 on [-2.5, 2.5] x [0, 4] with steps 0.05 (101 x 81 vertices),
    the lid faces of the 2D test problem, from rest; the first ``n_steps``
    steps of d_t."""
    diff_eq = ns.NavierStokesEquation(5000.0)
    mesh = ns.Mesh([(-2.5, 2.5), (0.0, 4.0)], [0.05, 0.05])
    vec = ns.vectorize_bc_function
    bcs = [
        (ns.DirichletBoundaryCondition(vec(lambda x, t: [1.0, 0.1, None, None]), is_static=True),
         ns.DirichletBoundaryCondition(vec(lambda x, t: [0.0, 0.0, None, None]), is_static=True)),
        (ns.DirichletBoundaryCondition(vec(lambda x, t: [0.0, 0.0, None, None]), is_static=True),
         ns.DirichletBoundaryCondition(vec(lambda x, t: [0.0, 0.0, None, None]), is_static=True)),
    ]
    cp = ns.ConstrainedProblem(diff_eq, mesh, bcs)
    ic = ns.ContinuousInitialCondition(cp, lambda x: np.zeros((len(x), 4)))
    return ns.InitialValueProblem(cp, (0.0, n_steps * d_t), ic)


# ---- supervised ML operator fixtures (shared by the golden generator, which
# runs the reference, and the tests, which run this package)

def sml_perturbation(t, y):
    """Perturbs an initial state with numpy's global generator (the draws
    depend on the caller's seeding and call order) and the start time."""
    return y + 0.05 * (1.0 + t) * np.random.random(y.shape)


class AffineModel:
    """A regression model with the fit / predict contract of a scikit-learn
    regressor: least squares on [x, 1] (deterministic)."""

    def fit(self, x, y):
        a = np.hstack([x, np.ones((len(x), 1))])
        self.coef_, *_ = np.linalg.lstsq(a, y, rcond=None)
        return self

    def predict(self, x):
        return np.hstack([x, np.ones((len(x), 1))]) @ self.coef_


def sml_diffusion_1d(ns, n=12, t_end=0.15):
    """1D diffusion on [0, 1], Dirichlet 0 / Neumann 0 ends, a sine bump."""
    diff_eq = ns.DiffusionEquation(1, 0.2)
    mesh = ns.Mesh([(0.0, 1.0)], [1.0 / n])
    lo = ns.DirichletBoundaryCondition(lambda x, t: np.zeros((len(x), 1)), is_static=True)
    hi = ns.NeumannBoundaryCondition(lambda x, t: np.zeros((len(x), 1)), is_static=True)
    cp = ns.ConstrainedProblem(diff_eq, mesh, [(lo, hi)])
    ic = ns.ContinuousInitialCondition(cp, lambda x: np.sin(np.pi * x[:, :1]) + 0.1)
    return ns.InitialValueProblem(cp, (0.0, t_end), ic)
