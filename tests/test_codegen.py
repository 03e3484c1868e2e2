"""Lowering and code generation (CPU: NVRTC compiles without a GPU)."""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import FDM_CASES
from pararealml_gb300 import _native, codegen
from pararealml_gb300.operators.fdm.numerical_integrator import integrator_kind
from pararealml_gb300.operators import fdm


def test_stage_invariance_detection():
    ch = problems.cahn_hilliard_2d(ns).constrained_problem
    assert codegen.is_stage_invariant(codegen.lower_problem(ch), codegen.RK4)
    dif = problems.diffusion_2d(ns, n=16).constrained_problem
    assert not codegen.is_stage_invariant(codegen.lower_problem(dif), codegen.RK4)
    sw = problems.shallow_water_2d(ns).constrained_problem
    assert not codegen.is_stage_invariant(codegen.lower_problem(sw), codegen.RK4)


def test_face_tables_follow_constraints():
    low = codegen.lower_problem(problems.mixed_bc_wave_2d(ns).constrained_problem)
    nx, ny = low.nx, low.ny
    # axis 0 lower face: Dirichlet on y_0 = sin(x_1), y_1 free
    assert np.allclose(low.dirichlet[0, 0, :ny], np.sin(low.coord_k1))
    assert np.all(np.isnan(low.dirichlet[0, 1, :ny]))
    # axis 1 lower face: Neumann on y_0 = 0.3 x_0 where x_0 <= 1, else free
    x0 = low.coord_k0
    want = np.where(x0 > 1.0, np.nan, 0.3 * x0)
    got = low.neumann[2, 0, :nx]
    assert np.array_equal(np.isnan(got), np.isnan(want))
    assert np.allclose(got[~np.isnan(got)], want[~np.isnan(want)])
    assert low.dir_mask & (1 << (0 * 2 + 0))
    assert not low.dir_mask & (1 << (0 * 2 + 1))


def test_unsupported_problems_are_rejected():
    with pytest.raises(NotImplementedError):
        integrator_kind(object())


def test_laplacian_rows_lower_as_right_hand_side_rows():
    """LHS.Y_LAPLACIAN rows: the step kernel stores their right-hand side at
    (t, y) like LHS.Y rows (the Jacobi solve replaces it), and no temporally
    blocked kernel is generated (a solve runs between every two steps)."""
    cp = ns.ConstrainedProblem(ns.NavierStokesEquation(), ns.Mesh([(0, 1), (0, 1)], [0.1, 0.1]),
                               [(ns.DirichletBoundaryCondition(lambda x, t: np.zeros((len(x), 4)), is_static=True),) * 2] * 2)
    low = codegen.lower_problem(cp)
    assert low.d_idx == (0,) and low.lap_idx == (1,) and low.y_idx == (1, 2, 3)
    assert low.mesh_dx == (0.1, 0.1) and len(low.axis_coords) == 2
    gen = codegen.generate_source(low, codegen.FORWARD_EULER, "f32")
    assert all(codegen.tile_steps(t) == 1 for t in gen.step_kernels)


def test_jacobi_coefficient_tables():
    """Reciprocals of the reference's divisors (numerical_differentiator.py:
    1115-1186), laid out as the C header's prml_jacobi_params describes."""
    from pararealml_gb300.engine import jacobi_coefficients

    assert np.isclose(jacobi_coefficients("CARTESIAN", (0.5, 0.25), None)[0], 1.0 / (2 / 0.25 + 2 / 0.0625))
    r, th, phi = np.array([1.0, 2.0, 3.0]), np.array([0.0, 0.5]), np.array([0.4, 0.8, 1.2, 1.6])
    pol = jacobi_coefficients("POLAR", (1.0, 0.5), (r, th))
    assert pol.shape == (9,)
    assert np.allclose(pol[:3], 1 / (2 * 1.0 * r)) and np.allclose(pol[3:6], 1 / r**2)
    assert np.allclose(pol[6:], 1 / (2 / 1.0 + 2 / (0.25 * r**2)))
    cyl = jacobi_coefficients("CYLINDRICAL", (1.0, 0.5, 0.2), (r, th, phi))
    assert np.allclose(cyl[6:], 1 / (2 / 1.0 + 2 / (0.25 * r**2) + 2 / 0.04))
    sph = jacobi_coefficients("SPHERICAL", (1.0, 0.5, 0.4), (r, th, phi))
    assert sph.shape == (3 + 3 + 4 + 4 + 12 + 12,)
    s2 = (r[:, None] * np.sin(phi)[None, :]) ** 2
    assert np.allclose(sph[:3], 1 / r) and np.allclose(sph[6:10], np.cos(phi))
    assert np.allclose(sph[10:14], 1 / (0.8 * np.sin(phi)))
    assert np.allclose(sph[14:26].reshape(3, 4), 1 / s2)
    den = 2 / 1.0 + 2 / (0.25 * s2) + 2 / (0.16 * r[:, None] ** 2)
    assert np.allclose(sph[26:].reshape(3, 4), 1 / den)


def test_time_dependent_boundary_tables():
    """Time-dependent conditions lower with presence bits wherever a condition
    of that kind exists, per-time tables from the problem's own constraint
    evaluation, and no stage invariance."""
    dyn = ns.DirichletBoundaryCondition(lambda x, t: np.zeros((len(x), 1)) + t + x[:, :1])
    neu = ns.NeumannBoundaryCondition(lambda x, t: np.full((len(x), 1), 2.0 * t))
    cp = ns.ConstrainedProblem(ns.DiffusionEquation(2), ns.Mesh([(0, 1), (0, 2)], [0.1, 0.1]), [(dyn, neu), (neu, dyn)])
    low = codegen.lower_problem(cp)
    assert low.dynamic and low.cp is cp
    # axis 0: lower Dirichlet (face 0), upper Neumann (face 1); axis 1: lower Neumann (face 2), upper Dirichlet (face 3)
    assert low.dir_mask == (1 << 0) | (1 << 3) and low.neu_mask == (1 << 1) | (1 << 2)
    d, n = codegen.face_tables_at(low, 0.75)
    nx, ny = low.nx, low.ny
    assert np.allclose(d[0, 0, :ny], 0.75 + 0.0)          # x_0 = 0 on the lower face of axis 0
    assert np.allclose(d[3, 0, :nx], 0.75 + low.coord_k0)  # x_0 varies along the upper face of axis 1
    assert np.allclose(n[1, 0, :ny], 1.5) and np.allclose(n[2, 0, :nx], 1.5)
    assert not codegen.is_stage_invariant(low, codegen.RK4)


def test_stencils_need_three_points():
    bc = ns.DirichletBoundaryCondition(lambda x, t: np.zeros((len(x), 1)), is_static=True)
    cp = ns.ConstrainedProblem(ns.DiffusionEquation(2), ns.Mesh([(0, 1), (0, 1)], [1.0, 0.5]), [(bc, bc)] * 2)
    low = codegen.lower_problem(cp)
    with pytest.raises(ValueError):
        codegen.generate_source(low, codegen.RK4, "f64")


def test_constants_printed_like_lambdify():
    low = codegen.lower_problem(problems.diffusion_2d(ns, n=8).constrained_problem)
    low.rhs = (low.rhs[0] * (1 / 3.0),)
    src = codegen.generate_source(low, codegen.FORWARD_EULER, "f64").source
    assert "T(0.333333333333333)" in src


@pytest.mark.parametrize("name", sorted(FDM_CASES))
@pytest.mark.parametrize("dtype", ["f32", "f32c", "f64"])
@pytest.mark.parametrize("kind", [codegen.FORWARD_EULER, codegen.EXPLICIT_MIDPOINT, codegen.RK4])
def test_shared_memory_layout_and_tma_boxes(name, dtype, kind):
    """Restates the step kernel's shared-memory layout and TMA geometry on the
    CPU: every staging buffer and the mbarriers are aligned, everything fits
    in the requested dynamic shared memory, boxes obey the TMA limits and
    every box's first column starts on a 16-byte boundary.  Temporally
    blocked kernels stage a halo as deep as their step count (and the lo
    planes of a compensated state)."""
    builder, kw, _, _ = FDM_CASES[name]
    low = codegen.lower_problem(builder(ns, **kw).constrained_problem)
    if low.x_dimension == 3 and dtype == "f32c":
        with pytest.raises(NotImplementedError):
            codegen.generate_source(low, kind, dtype)
        return
    gen = codegen.generate_source(low, kind, dtype)
    esize = 8 if dtype == "f64" else 4
    single_stage = codegen.stage_count(kind, gen.invariant, 0) == 1
    blocked = [t for t in gen.step_kernels if codegen.tile_steps(t) > 1]
    # temporal blocking exists for single-stage steps on 0-2D meshes without
    # LHS.Y_LAPLACIAN rows (their Jacobi solve runs between every two steps)
    assert bool(blocked) == (single_stage and low.x_dimension < 3 and not low.lap_idx)
    walk = [t for t in gen.step_kernels if codegen.is_walk(t)]
    # register-window kernels exist for single-stage steps on 2D meshes and
    # use no shared memory
    assert bool(walk) == (single_stage and low.x_dimension == 2)
    for tile in walk:
        assert gen.step_kernels[tile][1] == 0
        vw = 16 // esize
        assert tile[0] % 4 == 0 and tile[1] % (8 * vw) == 0 and tile[2] == 32 * (tile[1] // (8 * vw))
    staged = [(t, s) for t, (_, s) in gen.step_kernels.items() if not codegen.is_walk(t)]
    for mode, items in ((0, staged), (1, [(gen.rhs_kernel[2], gen.rhs_kernel[1])])):
        for tile, smem in items:
            k = codegen.tile_steps(tile)
            h = k if k > 1 else codegen.stage_count(kind, gen.invariant, mode)
            hx, hy = h, codegen.col_halo(h, esize)
            rx, ry = gen.box(tile, mode)
            assert (rx, ry) == (tile[0] + 2 * hx, tile[1] + 2 * hy)
            assert hy >= hx
            assert rx <= 256 and ry <= 256 and (ry * esize) % 16 == 0
            planes = gen.box_planes(tile) if mode == 0 else low.n_comp
            assert planes == (2 * low.n_comp if (dtype == "f32c" and k > 1) else low.n_comp)
            depth = gen.box_depth(tile, mode)
            if low.x_dimension == 3:
                assert depth == codegen.tile_planes(tile) + 2 * h and depth <= 256
                assert (tile[0] * tile[1] * codegen.tile_planes(tile)) % tile[2] == 0
            else:
                assert depth == 1
            buf_elems = ((planes * depth * rx * ry * esize + 127) // 128) * 128 // esize
            nstg = codegen.buffer_count(kind, gen.invariant, mode, tile) - 2
            if k > 1:
                assert nstg == (1 if k == 2 else 2)
            offsets = [j * buf_elems * esize for j in range(2 + nstg)]
            assert all(o % 128 == 0 for o in offsets)
            bar_off = (2 + nstg) * buf_elems * esize
            assert bar_off % 8 == 0
            assert 127 + bar_off + 16 <= smem <= codegen.SMEM_LIMIT
            tiles_x = (low.ny + tile[1] - 1) // tile[1]
            for tx in range(tiles_x):
                assert ((tx * tile[1] - hy) * esize) % 16 == 0
            assert tile[1] % (16 // esize) == 0
            if low.x_dimension < 3:
                assert (tile[0] * tile[1]) % tile[2] == 0
            assert k <= 8


def test_exact_division_switch():
    """Modules of the implicit integrators divide like numpy (EXACT_DIV);
    the switch is part of the source, so it gets its own cubin."""
    low = codegen.lower_problem(problems.diffusion_2d(ns, n=8).constrained_problem)
    plain = codegen.generate_source(low, codegen.FORWARD_EULER, "f64")
    exact = codegen.generate_source(low, codegen.FORWARD_EULER, "f64", exact_div=True)
    assert "EXACT_DIV = false" in plain.source and "EXACT_DIV = true" in exact.source
    assert plain.key != exact.key
    _native.jit_module(exact.source, exact.key, "--fmad=false")


def test_implicit_integrator_mirror():
    """Constructors and validation of numerical_integrator.py:135-248, and
    the settings read from this package's or the reference's objects."""
    from pararealml_gb300.operators.fdm.numerical_integrator import implicit_settings

    be = fdm.BackwardEulerMethod(1e-6, 7)
    cn = fdm.CrankNicolsonMethod(0.7, 1e-9, 11)
    assert implicit_settings(be) == {"a": 1.0, "tol": 1e-6, "max_iterations": 7, "crank_nicolson": False}
    assert implicit_settings(cn) == {"a": 0.7, "tol": 1e-9, "max_iterations": 11, "crank_nicolson": True}
    for bad in (lambda: fdm.BackwardEulerMethod(-1.0), lambda: fdm.BackwardEulerMethod(1e-8, 0),
                lambda: fdm.CrankNicolsonMethod(1.5)):
        with pytest.raises(ValueError):
            bad()
    assert integrator_kind(cn) == codegen.CRANK_NICOLSON


def _walk_accesses(nx, ny, pitch, esize, rows_per_thread, warps, grid):
    """Replays walk_body / walk_tile's index arithmetic and predicates for
    every thread of a launch: the (row, first column, width) of each global
    load and store it executes, and the vertices it stores."""
    vw = 16 // esize
    tx_rows, ty_cols = 4 * rows_per_thread, warps * 8 * vw
    tiles_x, tiles_y = -(-ny // ty_cols), -(-nx // tx_rows)
    loads, stores, stored = [], [], set()
    for t in range(tiles_x * tiles_y):  # one instance; the walk visits every tile once
        ty, tx = divmod(t, tiles_x)
        for wid in range(warps):
            ri, cw = ty * tx_rows, tx * ty_cols + wid * 8 * vw
            if cw >= ny:
                continue
            edge = ri < 2 or ri + tx_rows + 2 > nx or cw < 2 or cw + 8 * vw + 2 > ny
            for lane in range(32):
                q, g = lane >> 3, lane & 7
                gi0, gj0 = ri + q * rows_per_thread, cw + g * vw
                cols_in = gj0 < ny
                for r in range(rows_per_thread + 2):
                    gi = gi0 - 1 + r
                    row_in = (not edge) or (0 <= gi < nx)
                    if row_in and ((not edge) or cols_in):
                        loads.append((gi, gj0, vw))
                    if g == 0 and row_in and ((not edge) or (gj0 >= 1 and gj0 - 1 < ny)):
                        loads.append((gi, gj0 - 1, 1))
                    if g == 7 and row_in and ((not edge) or gj0 + vw < ny):
                        loads.append((gi, gj0 + vw, 1))
                for r in range(rows_per_thread):
                    gi = gi0 + r
                    if edge and gi >= nx:
                        break
                    if edge and not cols_in:
                        continue
                    if (not edge) or gj0 + vw <= ny:
                        stores.append((gi, gj0, vw))
                        stored.update((gi, gj0 + k) for k in range(vw))
                    else:
                        for k in range(vw):
                            if gj0 + k >= ny:
                                break
                            stores.append((gi, gj0 + k, 1))
                            stored.add((gi, gj0 + k))
    return loads, stores, stored


@pytest.mark.parametrize("esize", [4, 8])
@pytest.mark.parametrize("nx,ny", [(3, 3), (5, 40), (40, 5), (17, 33), (65, 65), (130, 257), (1025, 1025)])
def test_register_window_accesses_stay_inside_the_state(esize, nx, ny):
    """Every global access of the register-window kernel stays inside the
    rows of the mesh and the row pitch (no read of a neighbouring row or
    instance), 16-byte loads and stores start on 16-byte boundaries, and
    the stores cover each vertex of the mesh exactly once and nothing else
    (the row padding is never written)."""
    pitch = -(-ny // 32) * 32
    vw = 16 // esize
    for r_rows, warps in codegen.WALK_CONFIGS:
        if nx * ny > 70000 and (r_rows, warps) != (2, 4):
            continue
        loads, stores, stored = _walk_accesses(nx, ny, pitch, esize, r_rows, warps, 0)
        for gi, gj, width in loads + stores:
            assert 0 <= gi < nx, (gi, gj, width)
            assert 0 <= gj and gj + width <= pitch, (gi, gj, width)
            if width > 1:
                assert (gj * esize) % 16 == 0 and width == vw
        assert all(0 <= gi < nx and 0 <= gj < ny for gi, gj in stored)
        assert len(stored) == nx * ny
        assert sum(w for _, _, w in stores) == nx * ny
