"""GPU parity of the fused FDM kernels (needs a GB300).

Bars: float64 results match the reference's own outputs (golden fixtures)
and the CPU oracle to REL_F64 = 1e-12 relative L2; float32 results match the
float64 reference to REL_F32 = 5e-5 relative L2 (the FP32 path's stated
error on these problems).  Stencil known answers are the reference's own
differentiator/integrator test vectors, evaluated by the generated
right-hand-side kernel.
"""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import FDM_CASES, ORACLE_INTEGRATOR, is_implicit, load, make_integrator, rel_l2
from oracle import fdm as orc
from pararealml_gb300 import codegen
from pararealml_gb300.operators import fdm

pytestmark = pytest.mark.gpu

REL_F64 = 1e-12
REL_F32 = 5e-5
# The reference's cylindrical and spherical diffusion tests step at dt = 0.1,
# where RK4 amplifies the angular modes of the discrete Laplacian up to ~556
# times per step; they stay bounded only because the initial state 1 / r is
# exactly symmetric in the angles and every vertex rounds identically.  Any
# asymmetric rounding (float32 contracts multiply-adds differently in
# different code paths) grows by ~1e27 over 10 steps, so only float64 parity
# is defined for them.
UNSTABLE_SYMMETRIC = {"cylindrical_diffusion_rk4", "spherical_diffusion_rk4"}


@pytest.fixture(scope="module", autouse=True)
def _built():
    from pararealml_gb300 import _native

    _native.build()
    yield


def _op(integ, d_t, **kw):
    return fdm.FDMOperator(make_integrator(fdm, integ), fdm.ThreePointCentralDifferenceMethod(), d_t, **kw)


@pytest.mark.parametrize("name", sorted(FDM_CASES))
def test_f64_matches_reference(name):
    builder, kw, integ, d_t = FDM_CASES[name]
    gold = load(name)
    ivp = builder(ns, **kw)
    if is_implicit(integ):
        # start from the reference's own initial state: the secant's stop
        # test turns a one-ulp difference (Gaussian initial states go through
        # the host's libm exp, which rounds differently on aarch64 and x86)
        # into differences of the order of its tolerance
        cp = ivp.constrained_problem
        ivp = ns.InitialValueProblem(cp, ivp.t_interval, ns.DiscreteInitialCondition(cp, np.array(gold["y0"]), True))
    np.random.seed(problems.JACOBI_SEED)  # LHS.Y_LAPLACIAN: the reference's Jacobi estimates
    sol = _op(integ, d_t).solve(ivp)
    y = sol.discrete_y()
    assert y.shape[0] == int(gold["n_steps"])
    assert np.allclose(sol.t_coordinates[gold["steps"] - 1], gold["t"]) if "t" in gold else True
    assert rel_l2(y[gold["steps"] - 1], gold["y"]) < REL_F64


@pytest.mark.parametrize("name", sorted(FDM_CASES))
def test_f32_error_against_f64_reference(name):
    builder, kw, integ, d_t = FDM_CASES[name]
    if name in UNSTABLE_SYMMETRIC:
        pytest.skip("float32 parity is undefined for an unstable problem held by exact symmetry")
    if is_implicit(integ):
        pytest.skip("implicit integrators run in float64 only")
    gold = load(name)
    ivp = builder(ns, **kw)
    np.random.seed(problems.JACOBI_SEED)
    y = _op(integ, d_t, dtype="float32").solve(ivp).discrete_y()
    assert rel_l2(y[gold["steps"] - 1], gold["y"]) < REL_F32


@pytest.mark.parametrize("max_ctas", [0, 3])
@pytest.mark.parametrize("tile", list(codegen.TILE_CONFIGS + codegen.TB_CONFIGS))
@pytest.mark.parametrize(
    "name",
    ["cahn_hilliard_rk4", "shallow_water_rk4", "wave_mixed_rk4", "burgers_rk4", "diffusion_fe_65",
     "convdiff_1d_fe", "diffusion_midpoint"],
)
def test_every_tile_shape(name, tile, max_ctas):
    """Every tile shape; with max_ctas = 3 every CTA walks many tiles, so
    both TMA staging buffers and both mbarrier phases are exercised."""
    builder, kw, integ, d_t = FDM_CASES[name]
    gold = load(name)
    ivp = builder(ns, **kw)
    op = _op(integ, d_t)
    gen = codegen.generate_source(codegen.lower_problem(ivp.constrained_problem), op.integrator_kind, "f64")
    if tile not in gen.step_kernels:
        pytest.skip(f"tile {tile} does not fit in shared memory for this system")
    for dtype, tol in (("float64", REL_F64), ("float32", REL_F32)):
        y = _op(integ, d_t, tile=tile, max_ctas=max_ctas, dtype=dtype).solve(ivp).discrete_y()
        assert rel_l2(y[gold["steps"] - 1], gold["y"]) < tol


@pytest.mark.parametrize(
    "builder,kw,integ,d_t,steps",
    [
        ("cahn_hilliard_2d", dict(n=128, length=32.0, t_end=0.02), "RK4", 0.001, 20),
        ("shallow_water_2d", dict(n=96, length=64.0, t_end=1.0), "RK4", 0.05, 20),
        ("mixed_bc_wave_2d", dict(nx=131, ny=77, t_end=0.03), "RK4", 0.001, 30),
    ],
)
def test_larger_ragged_meshes_against_oracle(builder, kw, integ, d_t, steps):
    import problems

    ivp = getattr(problems, builder)(ns, **kw)
    cp = ivp.constrained_problem
    y0 = ivp.initial_condition.discrete_y_0(True)
    want = orc.fdm_solve(cp, y0, ivp.t_interval, d_t, ORACLE_INTEGRATOR[integ], keep="final", n_steps=steps)
    op = _op(integ, d_t, trajectory="final")
    got = op.solve(ns.InitialValueProblem(cp, (0.0, steps * d_t), ivp.initial_condition)).discrete_y()[-1]
    assert rel_l2(got, want) < REL_F64


def test_batched_instances_match_individual_solves():
    import problems
    import torch

    ivps = [problems.cahn_hilliard_2d(ns, n=40, length=10.0, seed=s) for s in (1, 2, 3)]
    cp = ivps[0].constrained_problem
    y0 = np.stack([ivp.initial_condition.discrete_y_0(True) for ivp in ivps])
    op = _op("RK4", 0.001)
    traj = op.solve_device(cp, torch.from_numpy(y0).cuda(), 0.0, 15, save_every=15)
    plan = op.plan(cp, 3)
    got = plan.unpack(traj[0], 3).cpu().numpy()
    for b in range(3):
        want = orc.fdm_solve(cp, y0[b], (0.0, 0.015), 0.001, "rk4", keep="final")
        assert rel_l2(got[b], want) < REL_F64


def test_strided_and_final_trajectories():
    builder, kw, integ, d_t = FDM_CASES["diffusion_rk4"]
    gold = load("diffusion_rk4")
    ivp = builder(ns, **kw)
    full = _op(integ, d_t).solve(ivp).discrete_y()
    strided = _op(integ, d_t, trajectory=5).solve(ivp)
    assert strided.discrete_y().shape[0] == full.shape[0] // 5
    assert np.array_equal(strided.discrete_y(), full[4::5])
    final = _op(integ, d_t, trajectory="final", keep_on_device=True).solve(ivp)
    assert final.device_y is not None
    assert np.array_equal(final.discrete_y()[-1], full[-1])
    assert rel_l2(full[-1], gold["y"][-1]) < REL_F64
    with pytest.raises(ValueError):
        _op(integ, d_t, trajectory=7).solve(ivp)


# ---- the reference's stencil known answers, through the RHS kernel
class SymbolEquation(ns.DifferentialEquation):
    def __init__(self, x_dim, y_dim, make):
        self._make = make
        super().__init__(x_dim, y_dim)

    @property
    def symbolic_equation_system(self):
        return ns.SymbolicEquationSystem(self._make(self._symbols))


def _bc(fn_by_coord, n_comp):
    """Neumann condition from a per-point function returning n_comp values (None = free)."""
    return ns.NeumannBoundaryCondition(
        lambda x, t: np.array([[np.nan if v is None else v for v in fn_by_coord(p)] for p in x], float).reshape(len(x), n_comp),
        is_static=True,
    )


def _free(n_comp):
    return _bc(lambda p: [None] * n_comp, n_comp)


def _rhs(diff_eq, mesh, bcs, y):
    import torch

    cp = ns.ConstrainedProblem(diff_eq, mesh, bcs)
    op = _op("ForwardEulerMethod", 1.0)
    plan = op.plan(cp, 1)
    s = plan.new_state(2)
    plan.pack_device(torch.from_numpy(np.ascontiguousarray(y[np.newaxis], dtype=np.float64)).cuda(), s[0])
    plan.rhs(s[0], s[1], 0.0)
    return plan.unpack(s[1], 1).cpu().numpy()[0]


Y3x3x2 = np.array(
    [
        [[2.0, 4.0], [4.0, 8.0], [-3.0, 2.0]],
        [[6.0, 4.0], [4.0, 4.0], [5.0, -1.0]],
        [[2.0, 6.0], [8.0, 2.0], [-7.0, 7.0]],
    ]
)


def test_kat_gradient_2d_constrained():
    mesh = ns.Mesh([(0.0, 4.0), (0.0, 2.0)], [2.0, 1.0])
    eq = SymbolEquation(2, 2, lambda s: [s.y_gradient[0, 0], s.y_gradient[1, 0]])
    lower = _bc(lambda p: [None, 9999.0 if p[1] == 1.0 else None], 2)
    upper = _bc(lambda p: [-9999.0 if p[1] != 1.0 else None, None], 2)
    got = _rhs(eq, mesh, [(lower, upper), (_free(2), _free(2))], Y3x3x2)
    exp = np.array(
        [
            [[1.5, 1.0], [1.0, 9999.0], [1.25, -0.25]],
            [[0.0, 0.5], [1.0, -1.5], [-1.0, 1.25]],
            [[-9999.0, -1.0], [-1.0, -1.0], [-9999.0, 0.25]],
        ]
    )
    assert np.allclose(got, exp, rtol=0, atol=1e-12)


def test_kat_hessian_2d_constrained():
    mesh = ns.Mesh([(0.0, 4.0), (0.0, 4.0)], [2.0, 2.0])
    eq = SymbolEquation(2, 2, lambda s: [s.y_hessian[0, 0, 0], s.y_hessian[1, 0, 0]])
    lower = _bc(lambda p: [None, -2.0 if p[1] < 3.0 else None], 2)
    upper = _bc(lambda p: [None, 0.0 if p[1] > 3.0 else None], 2)
    got = _rhs(eq, mesh, [(lower, upper), (_free(2), _free(2))], Y3x3x2)
    exp = np.array(
        [
            [[0.5, 2.0], [-1.0, 0.0], [2.75, -1.25]],
            [[-2.0, 0.5], [1.0, 0.5], [-5.0, 2.75]],
            [[0.5, -2.0], [-3.0, 0.0], [4.75, -4.0]],
        ]
    )
    assert np.allclose(got, exp, rtol=0, atol=1e-12)


def test_kat_hessian_1d_constrained_and_mixed():
    mesh = ns.Mesh([(0.0, 6.0)], [2.0])
    eq = SymbolEquation(1, 1, lambda s: [s.y_hessian[0, 0, 0]])
    got = _rhs(eq, mesh, [(_bc(lambda p: [0.0], 1), _free(1))], np.array([[2.0], [4.0], [-3.0], [-3.0]]))
    assert np.allclose(got, [[1.0], [-2.25], [1.75], [0.75]], rtol=0, atol=1e-12)

    mesh = ns.Mesh([(0.0, 2.0), (0.0, 1.0)], [1.0, 0.5])
    eq = SymbolEquation(2, 1, lambda s: [s.y_hessian[0, 0, 1]])
    y = np.array([[[2.0], [4.0], [-3.0]], [[6.0], [4.0], [5.0]], [[2.0], [8.0], [-7.0]]])
    got = _rhs(eq, mesh, [(_free(1), _free(1))] * 2, y)
    exp = np.array([[[2.0], [-0.5], [-2.0]], [[2.0], [-2.0], [-2.0]], [[-2.0], [0.5], [2.0]]])
    assert np.allclose(got, exp, rtol=0, atol=1e-12)


def test_kat_laplacian_and_divergence():
    mesh = ns.Mesh([(0.0, 4.0), (0.0, 2.0)], [2.0, 1.0])
    eq = SymbolEquation(2, 2, lambda s: [s.y_laplacian[0], s.y_laplacian[1]])
    y = np.array(
        [
            [[2.0, 4.0], [4.0, 8.0], [2.0, 4.0]],
            [[6.0, 4.0], [4.0, 4.0], [10.0, -4.0]],
            [[2.0, 6.0], [8.0, 2.0], [-2.0, 4.0]],
        ]
    )
    exp = np.array(
        [
            [[0.5, -1.0], [-5.0, -11.0], [1.5, -3.0]],
            [[-10.0, -3.5], [9.0, -7.5], [-21.0, 16.0]],
            [[4.5, -12.0], [-19.0, 6.0], [15.5, -9.0]],
        ]
    )
    assert np.allclose(_rhs(eq, mesh, [(_free(2), _free(2))] * 2, y), exp, rtol=0, atol=1e-12)

    mesh = ns.Mesh([(0.0, 2.0), (0.0, 4.0)], [1.0, 2.0])
    eq = SymbolEquation(2, 2, lambda s: [s.y_divergence[0, 1], s.y_gradient[1, 1]])
    got = _rhs(eq, mesh, [(_free(2), _free(2))] * 2, Y3x3x2)
    exp_div = np.array([[[5.0], [1.5], [0.5]], [[1.0], [0.75], [-3.0]], [[-2.5], [-1.75], [-3.0]]])
    assert np.allclose(got[..., :1], exp_div, rtol=0, atol=1e-12)
    exp_grad = orc.gradient(Y3x3x2[..., 1:], (1.0, 2.0), 1)
    assert np.allclose(got[..., 1:], exp_grad, rtol=0, atol=1e-12)


def test_kat_integrators_on_odes():
    class Eq(ns.DifferentialEquation):
        def __init__(self, make):
            self._make = make
            super().__init__(0, 1)

        @property
        def symbolic_equation_system(self):
            return ns.SymbolicEquationSystem(self._make(self._symbols))

    fe_eq = Eq(lambda s: [5.0 * s.y[0] + s.t**2])
    cp = ns.ConstrainedProblem(fe_eq)
    ivp = ns.InitialValueProblem(cp, (1.0, 1.5), ns.ConstantInitialCondition(cp, [1.0]))
    assert np.allclose(_op("ForwardEulerMethod", 0.5).solve(ivp).discrete_y(), [[4.0]])

    rk_eq = Eq(lambda s: [2.0 * s.y[0] + 1.0])
    cp = ns.ConstrainedProblem(rk_eq)
    ivp = ns.InitialValueProblem(cp, (1.0, 2.0), ns.ConstantInitialCondition(cp, [0.0]))
    assert np.allclose(_op("RK4", 1.0).solve(ivp).discrete_y(), [[3.0]])


def test_rk4_with_dirichlet_ends():
    class Eq(ns.DifferentialEquation):
        def __init__(self):
            super().__init__(1, 1)

        @property
        def symbolic_equation_system(self):
            return ns.SymbolicEquationSystem([2 * self._symbols.y[0] + 1])

    mesh = ns.Mesh([(0.0, 7.0)], [1.0])
    bc = ns.DirichletBoundaryCondition(lambda x, t: np.zeros((len(x), 1)), is_static=True)
    cp = ns.ConstrainedProblem(Eq(), mesh, [(bc, bc)])
    ivp = ns.InitialValueProblem(cp, (1.0, 2.0), ns.ConstantInitialCondition(cp, [0.0]))
    got = _op("RK4", 1.0).solve(ivp).discrete_y()[-1]
    exp = np.full((8, 1), 3.0)
    exp[0] = exp[-1] = 0.0
    assert np.allclose(got, exp)


REL_F32C = 1e-7
# The reference's own dynamic-boundary problem takes steps whose increment
# is as large as the state (D dt / dx^2 = 0.75): the compensated state then
# only removes the rounding of the update, not the float32 rounding of the
# right-hand side itself (~6e-8 of the increment per step, 20 steps).
# Time-dependent Dirichlet values (here sin(x + 3t) along a face) sit in
# float32 tables, so each constrained vertex carries float32 rounding into
# every stage of every step.
REL_F32C_LARGE_STEPS = {"diffusion_1d_dynamic_rk4": 1e-5, "wave_dynamic_rk4": 3e-7}
# LHS.Y_LAPLACIAN rows are solved by a plain float32 Jacobi loop (their
# remainder planes stay zero), which carries float32 rounding of the solved
# rows into every step.
REL_F32C_LARGE_STEPS.update({name: 1e-6 for name in FDM_CASES if name.startswith(("jacobi_", "navier_"))})


@pytest.mark.parametrize("name", sorted(FDM_CASES))
def test_compensated_float32_against_reference(name):
    """float32 arithmetic with a float32 remainder per state value (exact
    two-sum updates): the accumulated rounding of the updates is carried, so
    the result stays within REL_F32C of the float64 reference (small steps)."""
    builder, kw, integ, d_t = FDM_CASES[name]
    gold = load(name)
    ivp = builder(ns, **kw)
    if ivp.constrained_problem.differential_equation.x_dimension == 3:
        pytest.skip("compensated float32 is not available on 3D meshes")
    if is_implicit(integ):
        pytest.skip("implicit integrators run in float64 only")
    np.random.seed(problems.JACOBI_SEED)
    y = _op(integ, d_t, dtype="float32c").solve(ivp).discrete_y()
    assert rel_l2(y[gold["steps"] - 1], gold["y"]) < REL_F32C_LARGE_STEPS.get(name, REL_F32C)


BLOCKED_CASES = {
    "cahn_hilliard_rk4": ("cahn_hilliard_2d", dict(n=69, length=17.25, t_end=0.021), "RK4", 1e-3),
    "wave_mixed_fe": ("mixed_bc_wave_2d", dict(nx=131, ny=77, t_end=0.021), "ForwardEulerMethod", 1e-3),
    "burgers_cauchy_fe": ("burgers_2d", dict(n=50, t_end=0.0021), "ForwardEulerMethod", 1e-4),
    "convdiff_1d_fe": ("convection_diffusion_1d", dict(n=300, t_end=0.021), "ForwardEulerMethod", 1e-3),
    "wave_dynamic_fe": ("dynamic_bc_wave_2d", dict(nx=40, ny=33, t_end=0.021), "ForwardEulerMethod", 1e-3),
}


@pytest.mark.parametrize("dtype", ["float64", "float32", "float32c"])
@pytest.mark.parametrize("tile", list(codegen.TB_CONFIGS))
@pytest.mark.parametrize("name", sorted(BLOCKED_CASES))
def test_temporally_blocked_steps_equal_single_steps(name, tile, dtype):
    """Kernels that take K steps per launch (halo K deep, the ring values
    recomputed on chip) against one step per launch on the same problem, 21
    steps (not a multiple of K: the last launch takes fewer steps), full and
    every-third-step trajectories, CTAs walking many tiles.  Bars: float64 bit
    for bit (the blocked kernel evaluates the same expressions on the same
    values, and float64 modules are built without FMA contraction); float32
    within 1e-6 and compensated float32 within 1e-7 relative L2 (float32
    modules contract multiply-adds, and the compiler may contract the blocked
    and single-step copies of an expression differently)."""
    import problems

    builder, kw, integ, d_t = BLOCKED_CASES[name]
    ivp = getattr(problems, builder)(ns, **kw)
    op = _op(integ, d_t)
    code = {"float64": "f64", "float32": "f32", "float32c": "f32c"}[dtype]
    gen = codegen.generate_source(codegen.lower_problem(ivp.constrained_problem), op.integrator_kind, code)
    if tile not in gen.step_kernels:
        pytest.skip(f"tile {tile} does not fit in shared memory for this system")
    single = (32, 32, 256)
    for traj in ("full", 3):
        ref = _op(integ, d_t, dtype=dtype, tile=single, trajectory=traj).solve(ivp).discrete_y()
        got = _op(integ, d_t, dtype=dtype, tile=tile, trajectory=traj, max_ctas=3).solve(ivp).discrete_y()
        assert got.shape == ref.shape and ref.shape[0] == (21 if traj == "full" else 7)
        if dtype == "float64":
            assert np.array_equal(got, ref), float(np.max(np.abs(got - ref)))
        else:
            assert rel_l2(got, ref) < (1e-6 if dtype == "float32" else 1e-7)


@pytest.mark.parametrize("every", [1, 3])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_streamed_host_trajectory_equals_device_trajectory(dtype, every):
    """``solve_into`` streams the trajectory to a pinned host buffer in
    chunks (here 4 saved steps per chunk, a ragged last chunk) while the next
    chunk computes; the result equals ``solve`` bit for bit."""
    import torch

    import problems

    ivp = problems.cahn_hilliard_2d(ns, n=69, length=17.25, t_end=0.021)
    ref = _op("RK4", 1e-3, dtype=dtype, trajectory=every if every > 1 else "full").solve(ivp)
    y_ref = ref.discrete_y()
    out = torch.empty(y_ref.shape, dtype=torch.float64, pin_memory=True)
    out.fill_(np.nan)
    op = _op("RK4", 1e-3, dtype=dtype, trajectory=every if every > 1 else "full")
    sol = op.solve_into(ivp, out, chunk_saves=4)
    assert np.array_equal(sol.discrete_y(), y_ref)
    assert np.array_equal(sol.t_coordinates, ref.t_coordinates)


def test_streamed_trajectory_into_a_huge_page_buffer():
    """The same stream into a ``PinnedHostBuffer`` (anonymous mapping on huge
    pages, registered with CUDA): CUDA sees it as pinned, the result equals
    ``solve`` bit for bit, and closing it releases the mapping."""
    import problems
    from pararealml_gb300.hostmem import PinnedHostBuffer

    ivp = problems.cahn_hilliard_2d(ns, n=69, length=17.25, t_end=0.021)
    y_ref = _op("RK4", 1e-3, dtype="float64", trajectory="full").solve(ivp).discrete_y()
    with PinnedHostBuffer(y_ref.shape) as buf:
        assert buf.tensor.is_pinned() and buf.nbytes == y_ref.nbytes
        buf.tensor.fill_(np.nan)
        sol = _op("RK4", 1e-3, dtype="float64", trajectory="full").solve_into(ivp, buf.tensor, chunk_saves=5)
        assert np.array_equal(sol.discrete_y(), y_ref)
    assert buf.tensor is None and buf._ptr is None


def _forced_heat_equation():
    """dy/dt = 0.3 lap(y) + sin(3 t) x_0 - 0.2 x_1 y: a right-hand side that
    reads the time and both vertex coordinates."""
    import sympy as sp

    class ForcedHeat(ns.DifferentialEquation):
        def __init__(self):
            super().__init__(2, 1)

        @property
        def symbolic_equation_system(self):
            s = self.symbols
            return ns.SymbolicEquationSystem(
                [0.3 * s.y_laplacian[0] + sp.sin(3 * s.t) * s.x[0] - 0.2 * s.x[1] * s.y[0]]
            )

    return ForcedHeat()


@pytest.mark.parametrize("integ", ["RK4", "ForwardEulerMethod"])
def test_time_and_coordinate_dependent_rhs_against_oracle(integ):
    """Time and coordinates enter the generated kernel (the float64 path in
    double, the float32 path through host-rounded float copies); mixed
    Dirichlet / Neumann faces, a start time away from zero, 37 steps.
    Bars: float64 within 1e-12, float32 within 5e-5 relative L2 of the oracle."""
    de = _forced_heat_equation()
    mesh = ns.Mesh([(-1.0, 2.0), (0.5, 3.0)], [3.0 / 45, 2.5 / 38])
    bc_d = ns.DirichletBoundaryCondition(lambda x, t: np.full((len(x), 1), 0.2), is_static=True)
    bc_n = ns.NeumannBoundaryCondition(lambda x, t: np.full((len(x), 1), -0.1), is_static=True)
    cp = ns.ConstrainedProblem(de, mesh, [(bc_d, bc_n), (bc_n, bc_d)])
    ic = ns.GaussianInitialCondition(cp, [(np.array([0.5, 1.7]), 0.3 * np.eye(2))], [1.0])
    d_t = 1e-3
    ivp = ns.InitialValueProblem(cp, (0.25, 0.25 + 37 * d_t), ic)
    y0 = ivp.initial_condition.discrete_y_0(True)
    want = orc.fdm_solve(cp, y0, ivp.t_interval, d_t, ORACLE_INTEGRATOR[integ], keep="final", n_steps=37)
    for dtype, tol in (("float64", REL_F64), ("float32", REL_F32)):
        got = _op(integ, d_t, dtype=dtype, trajectory="final").solve(ivp).discrete_y()[-1]
        assert rel_l2(got, want) < tol, dtype


def test_reference_dynamic_boundary_condition_assertions():
    """The reference's own time-dependent boundary test
    (tests/operators/fdm/test_fdm_operator.py:293-319), float64 and float32."""
    import problems

    ivp = problems.dynamic_bc_diffusion_1d(ns)
    for dtype in ("float64", "float32"):
        sol = _op("RK4", 0.5, dtype=dtype).solve(ivp)
        y = sol.discrete_y()
        assert sol.vertex_oriented and sol.d_t == 0.5
        assert y.shape == (20, 11, 1)
        assert sol.discrete_y(False).shape == (20, 10, 1)
        assert np.isclose(y[0, -1, 0], 0.1)
        assert np.isclose(y[-1, -1, 0], 2.0)


@pytest.mark.parametrize("max_ctas", [0, 3])
@pytest.mark.parametrize("tile", list(codegen.TILE_CONFIGS_3D))
@pytest.mark.parametrize("name", ["cahn_hilliard_3d_rk4", "diffusion_3d_rk4", "diffusion_3d_fe", "spherical_diffusion_rk4",
                                  "cylindrical_vector_fe"])
def test_every_3d_tile_shape(name, tile, max_ctas):
    """3D meshes (planes x rows x columns tiles, 5D TMA boxes, six faces):
    every tile shape against the reference's goldens; with max_ctas = 3 each
    CTA walks many tiles.  Bars: float64 1e-12, float32 5e-5."""
    builder, kw, integ, d_t = FDM_CASES[name]
    gold = load(name)
    ivp = builder(ns, **kw)
    op = _op(integ, d_t)
    gen = codegen.generate_source(codegen.lower_problem(ivp.constrained_problem), op.integrator_kind, "f64")
    if tile not in gen.step_kernels:
        pytest.skip(f"tile {tile} does not fit in shared memory for this system")
    legs = (("float64", REL_F64),) if name in UNSTABLE_SYMMETRIC else (("float64", REL_F64), ("float32", REL_F32))
    for dtype, tol in legs:
        y = _op(integ, d_t, tile=tile, max_ctas=max_ctas, dtype=dtype).solve(ivp).discrete_y()
        assert rel_l2(y[gold["steps"] - 1], gold["y"]) < tol, dtype


def test_reference_3d_pde_assertions():
    """The reference's own 3D test (tests/operators/fdm/
    test_fdm_operator.py:173-197): shapes of a 100-step solve."""
    import problems

    ivp = problems.cahn_hilliard_3d(ns, t_end=5.0)
    sol = _op("RK4", 0.05).solve(ivp)
    assert sol.vertex_oriented and sol.d_t == 0.05
    assert sol.discrete_y().shape == (100, 11, 6, 6, 2)
    assert sol.discrete_y(False).shape == (100, 10, 5, 5, 2)
    assert np.all(np.isfinite(sol.discrete_y()))


@pytest.mark.parametrize("system,shape", [("POLAR", (50, 6, 11, 3)), ("CYLINDRICAL", (50, 6, 11, 3, 1)),
                                          ("SPHERICAL", (50, 6, 11, 5, 1))])
def test_reference_curvilinear_pde_assertions(system, shape):
    """The reference's own polar / cylindrical / spherical tests
    (tests/operators/fdm/test_fdm_operator.py:200-290): 50 RK4 steps of 0.1,
    solution shapes, finite values."""
    import problems

    if system == "POLAR":
        ivp = problems.polar_shallow_water(ns, t_end=5.0)
    else:
        ivp = problems.curvilinear_diffusion_3d(ns, system=system, t_end=5.0)
    sol = _op("RK4", 0.1).solve(ivp)
    y = sol.discrete_y()
    assert sol.vertex_oriented and sol.d_t == 0.1
    assert y.shape == shape
    assert np.all(np.isfinite(y))
