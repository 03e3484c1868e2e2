"""Generates the golden fixtures by running the reference PararealML itself.

Run from the repository root where the reference source tree is available:

    python tests/golden/make_golden.py [case ...]

It imports the unmodified reference through ``oracle/refshim.py`` (matplotlib
stubs, ``np.product`` alias and a thread-per-rank fake ``mpi4py``), solves
each case in ``CASES`` with the reference's own ``FDMOperator`` /
``PararealOperator`` and stores the initial state and selected trajectory
steps in ``tests/golden/<case>.npz``.  The problems come from
``tests/problems.py`` so the GPU tests can rebuild them bit-identically
with this package's classes.
"""

from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle import refshim  # noqa: E402
import problems  # noqa: E402

# case name -> (builder, builder kwargs, integrator, d_t, steps to keep (1-based; -1 = last))
CASES = {
    "diffusion_fe_65": (problems.diffusion_2d, dict(n=64, t_end=2.0), "ForwardEulerMethod", 0.0025, [1, 10, 100, 400, -1]),
    "diffusion_rk4": (problems.diffusion_2d, dict(n=32, t_end=0.5), "RK4", 0.01, [1, 7, -1]),
    "diffusion_midpoint": (problems.diffusion_2d, dict(n=32, t_end=0.5), "ExplicitMidpointMethod", 0.01, [1, -1]),
    "cahn_hilliard_rk4": (problems.cahn_hilliard_2d, dict(n=32, length=8.0, t_end=0.05), "RK4", 0.001, [1, 2, -1]),
    "cahn_hilliard_fe": (problems.cahn_hilliard_2d, dict(n=32, length=8.0, t_end=0.05), "ForwardEulerMethod", 0.001, [1, -1]),
    "shallow_water_rk4": (problems.shallow_water_2d, dict(n=32, length=64.0, t_end=2.0), "RK4", 0.1, [1, 5, -1]),
    "wave_mixed_rk4": (problems.mixed_bc_wave_2d, dict(nx=24, ny=20, t_end=0.1), "RK4", 0.005, [1, -1]),
    "wave_mixed_midpoint": (problems.mixed_bc_wave_2d, dict(nx=24, ny=20, t_end=0.1), "ExplicitMidpointMethod", 0.005, [1, -1]),
    "burgers_rk4": (problems.burgers_2d, dict(n=24, t_end=0.05), "RK4", 0.001, [1, -1]),
    "convdiff_1d_fe": (problems.convection_diffusion_1d, dict(n=50, t_end=0.2), "ForwardEulerMethod", 0.01, [1, -1]),
    "population_growth_rk4": (problems.population_growth, dict(t_end=1.0), "RK4", 0.01, [1, -1]),
    "diffusion_1d_dynamic_rk4": (problems.dynamic_bc_diffusion_1d, dict(), "RK4", 0.5, [1, 2, -1]),
    "wave_dynamic_rk4": (problems.dynamic_bc_wave_2d, dict(), "RK4", 0.002, [1, 7, -1]),
    "wave_dynamic_fe": (problems.dynamic_bc_wave_2d, dict(), "ForwardEulerMethod", 0.001, [1, 13, -1]),
    "wave_dynamic_midpoint": (problems.dynamic_bc_wave_2d, dict(), "ExplicitMidpointMethod", 0.002, [1, -1]),
    "cahn_hilliard_3d_rk4": (problems.cahn_hilliard_3d, dict(), "RK4", 0.05, [1, 5, -1]),
    "diffusion_3d_rk4": (problems.diffusion_3d_mixed, dict(), "RK4", 0.001, [1, 7, -1]),
    "diffusion_3d_fe": (problems.diffusion_3d_mixed, dict(), "ForwardEulerMethod", 0.0005, [1, -1]),
    "polar_shallow_water_rk4": (problems.polar_shallow_water, dict(), "RK4", 0.1, [1, 4, -1]),
    "cylindrical_diffusion_rk4": (problems.curvilinear_diffusion_3d, dict(system="CYLINDRICAL"), "RK4", 0.1, [1, -1]),
    "spherical_diffusion_rk4": (problems.curvilinear_diffusion_3d, dict(system="SPHERICAL"), "RK4", 0.1, [1, -1]),
    "spherical_vector_rk4": (problems.curvilinear_vector_field, dict(system="SPHERICAL"), "RK4", 0.001, [1, -1]),
    "cylindrical_vector_fe": (problems.curvilinear_vector_field, dict(system="CYLINDRICAL"), "ForwardEulerMethod", 0.0005, [1, -1]),
    "navier_stokes_rk4": (problems.navier_stokes_2d, dict(), "RK4", 0.25, [1, 5, 20, -1]),
    "jacobi_cartesian_1d_rk4": (problems.jacobi_system, dict(system="CARTESIAN", dims=1), "RK4", 0.005, [1, 2, -1]),
    "jacobi_cartesian_2d_rk4": (problems.jacobi_system, dict(system="CARTESIAN", dims=2), "RK4", 0.005, [1, 2, -1]),
    "jacobi_cartesian_3d_rk4": (problems.jacobi_system, dict(system="CARTESIAN", dims=3), "RK4", 0.005, [1, 2, -1]),
    "jacobi_polar_rk4": (problems.jacobi_system, dict(system="POLAR", dims=2), "RK4", 0.005, [1, 2, -1]),
    "jacobi_cylindrical_rk4": (problems.jacobi_system, dict(system="CYLINDRICAL", dims=3), "RK4", 0.005, [1, 2, -1]),
    "jacobi_spherical_rk4": (problems.jacobi_system, dict(system="SPHERICAL", dims=3), "RK4", 0.005, [1, 2, -1]),
    "jacobi_dynamic_fe": (problems.jacobi_system, dict(system="CARTESIAN", dims=2, dynamic=True), "ForwardEulerMethod", 0.005, [1, 2, -1]),
    "diffusion_be": (problems.diffusion_2d, dict(n=32, t_end=0.1), "BackwardEulerMethod", 0.01, [1, 5, -1]),
    "cahn_hilliard_cn": (problems.cahn_hilliard_2d, dict(n=32, length=8.0, t_end=0.01), "CrankNicolsonMethod", 0.001, [1, -1]),
    "cahn_hilliard_cn07": (problems.cahn_hilliard_2d, dict(n=32, length=8.0, t_end=0.01), "CrankNicolsonMethod:0.7", 0.001, [1, -1]),
    "wave_dynamic_be": (problems.dynamic_bc_wave_2d, dict(), "BackwardEulerMethod", 0.002, [1, 7, -1]),
    "convdiff_1d_cn": (problems.convection_diffusion_1d, dict(n=50, t_end=0.2), "CrankNicolsonMethod", 0.01, [1, -1]),
    "diffusion_3d_be": (problems.diffusion_3d_mixed, dict(), "BackwardEulerMethod", 0.002, [1, -1]),
    "navier_stokes_cn": (problems.navier_stokes_2d, dict(t_end=2.0), "CrankNicolsonMethod", 0.25, [1, -1]),
}

# Parareal cases: (builder, kwargs, fine integ, fine dt, coarse integ, coarse dt, ranks, tol, max_it, keep)
PARAREAL_CASES = {
    "parareal_diffusion": (problems.diffusion_2d, dict(n=32, t_end=1.0), "RK4", 0.005, "ForwardEulerMethod", 0.0125, 4, 1e-6, 100, [1, 50, 51, -1]),
    "parareal_cahn_hilliard_maxit": (problems.cahn_hilliard_2d, dict(n=24, length=6.0, t_end=0.08), "RK4", 0.001, "ForwardEulerMethod", 0.004, 4, 1e-9, 2, [1, 20, 21, -1]),
    # time-dependent boundary conditions: every rank's sub-IVP starts at its
    # own slice time (the reference's own dynamic-boundary test problem, and
    # the 2D wave with time-dependent, partly masked Dirichlet/Neumann faces)
    "parareal_dynamic_diffusion_1d": (problems.dynamic_bc_diffusion_1d, dict(), "RK4", 0.1, "ForwardEulerMethod", 0.25, 4, 1e-6, 100, [1, 25, 26, -1]),
    "parareal_dynamic_wave": (problems.dynamic_bc_wave_2d, dict(t_end=0.04), "RK4", 0.001, "ForwardEulerMethod", 0.0025, 4, 1e-6, 100, [1, 10, 11, -1]),
    # implicit fine and coarse operators (element-wise secant solves per step)
    "parareal_implicit_diffusion": (problems.diffusion_2d, dict(n=16, t_end=0.2), "CrankNicolsonMethod", 0.01, "BackwardEulerMethod", 0.05, 4, 1e-6, 100, [1, 5, 6, -1]),
}


def main() -> None:
    pr = refshim.import_reference()
    import pararealml.operators.fdm as fdm
    from pararealml.operators.parareal import PararealOperator

    os.makedirs(HERE, exist_ok=True)
    only = set(sys.argv[1:])  # optional case names: regenerate just those
    for name, (builder, kw, integ, d_t, keep) in CASES.items():
        if only and name not in only:
            continue
        t0 = time.time()
        ivp = builder(pr, **kw)
        iname, _, iargs = integ.partition(":")  # e.g. "CrankNicolsonMethod:0.7"
        integrator = getattr(fdm, iname)(*[float(v) for v in iargs.split(",") if v])
        op = fdm.FDMOperator(integrator, fdm.ThreePointCentralDifferenceMethod(), d_t)
        # LHS.Y_LAPLACIAN solves draw their initial estimates from numpy's
        # global generator; the GPU tests seed it the same way
        np.random.seed(problems.JACOBI_SEED)
        sol = op.solve(ivp)
        y = sol.discrete_y()
        steps = [len(y) if s == -1 else s for s in keep]
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            y0=ivp.initial_condition.discrete_y_0(True),
            steps=np.array(steps),
            y=y[np.array(steps) - 1],
            t=sol.t_coordinates[np.array(steps) - 1],
            n_steps=len(y),
        )
        print(f"{name}: {len(y)} steps, {time.time() - t0:.2f}s")

    for name, (builder, kw, fi, fdt, gi, gdt, ranks, tol, max_it, keep) in PARAREAL_CASES.items():
        if only and name not in only:
            continue
        t0 = time.time()
        ivp = builder(pr, **kw)
        f = fdm.FDMOperator(getattr(fdm, fi)(), fdm.ThreePointCentralDifferenceMethod(), fdt)
        g = fdm.FDMOperator(getattr(fdm, gi)(), fdm.ThreePointCentralDifferenceMethod(), gdt)
        op = PararealOperator(f, g, tol, max_it)
        sols = refshim.run_ranks(ranks, lambda: op.solve(ivp))
        y = sols[0].discrete_y()
        for other in sols[1:]:
            assert np.array_equal(other.discrete_y(), y)
        steps = [len(y) if s == -1 else s for s in keep]
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            y0=ivp.initial_condition.discrete_y_0(True),
            steps=np.array(steps),
            y=y[np.array(steps) - 1],
            n_steps=len(y),
            ranks=ranks,
        )
        print(f"{name}: {len(y)} steps on {ranks} ranks, {time.time() - t0:.2f}s")


def solution_case() -> None:
    """``Solution.y`` (linear and nearest interpolation at scattered points),
    ``discrete_y(vertex_oriented=False)`` and ``Solution.diff`` of the
    reference on two solves of one problem with different time steps
    (pararealml/solution.py:114-258)."""
    pr = refshim.import_reference()
    import pararealml.operators.fdm as fdm

    ivp = problems.diffusion_2d(pr, n=16, t_end=0.2)
    fe = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.01).solve(ivp)
    rk = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.02).solve(ivp)
    x = np.random.default_rng(17).uniform(-0.5, 10.5, (5, 3, 2))  # a few points outside the mesh too
    diff = fe.diff([rk])
    np.savez_compressed(
        os.path.join(HERE, "solution_interp_diff.npz"),
        y0=ivp.initial_condition.discrete_y_0(True),
        y_fe=fe.discrete_y(), y_rk=rk.discrete_y(), t_fe=fe.t_coordinates, t_rk=rk.t_coordinates,
        x=x, y_linear=fe.y(x), y_nearest=fe.y(x, "nearest"), cells=fe.discrete_y(False),
        diff_t=diff.matching_time_points, diff_0=diff.differences[0],
    )
    print("solution_interp_diff: done")


# SupervisedMLOperator data generation cases: name -> (problem builder,
# builder kwargs, operator kwargs, generate_data kwargs)
SML_CASES = {
    "ar": ("sml_diffusion_1d", {}, dict(vertex_oriented=True), dict(iterations=3, seeds=[5])),
    "ar_iso": ("sml_diffusion_1d", {}, dict(vertex_oriented=True), dict(iterations=3, seeds=[6],
                                                                       isolate_perturbations=True)),
    "ar_dt": ("sml_diffusion_1d", {}, dict(vertex_oriented=True, input_d_t=True), dict(iterations=2, seeds=[7])),
    "ar_tv": ("sml_diffusion_1d", {}, dict(vertex_oriented=True, time_variant=True), dict(iterations=2, seeds=[9])),
    "tv": ("sml_diffusion_1d", {}, dict(vertex_oriented=True, auto_regressive=False, time_variant=True),
           dict(iterations=3, seeds=[8])),
    "jobs2": ("sml_diffusion_1d", {}, dict(vertex_oriented=True), dict(iterations=3, n_jobs=2, seeds=[10, 11])),
    "ar_2d": ("diffusion_2d", dict(n=6, t_end=0.15), dict(vertex_oriented=True), dict(iterations=2, seeds=[12])),
    "iso_2d_cells": ("diffusion_2d", dict(n=6, t_end=0.15), dict(vertex_oriented=False),
                     dict(iterations=2, seeds=[13], isolate_perturbations=True)),
}
SML_D_T, SML_ORACLE_D_T = 0.05, 0.01


def sml_case() -> None:
    """``SupervisedMLOperator.generate_data`` / ``fit_model`` / ``solve`` of
    the reference (pararealml/operators/ml/supervised/
    supervised_ml_operator.py) with its own RK4 FDMOperator as the oracle and
    ``problems.sml_perturbation`` (numpy's global generator, seeded per job
    by the method itself), then a least-squares ``problems.AffineModel``
    fitted on the first case's data (split under np.random.seed(3)) and
    applied auto-regressively by ``solve``."""
    pr = refshim.import_reference()
    sml = refshim.import_supervised_ml_operator()
    import pararealml.operators.fdm as fdm

    oracle = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), SML_ORACLE_D_T)
    out = {}
    for name, (builder, kw, op_kw, gen_kw) in SML_CASES.items():
        ivp = getattr(problems, builder)(pr, **kw)
        op = sml.SupervisedMLOperator(SML_D_T, **op_kw)
        x, y = op.generate_data(ivp, oracle, perturbation_function=problems.sml_perturbation, **gen_kw)
        out[f"{name}_x"], out[f"{name}_y"] = x, y
        print(f"sml {name}: inputs {x.shape}, targets {y.shape}")
    ivp = problems.sml_diffusion_1d(pr)
    op = sml.SupervisedMLOperator(SML_D_T, True)
    np.random.seed(3)
    train, test = op.fit_model(problems.AffineModel(), (out["ar_x"], out["ar_y"]), test_size=0.25)
    out["fit_scores"] = np.array([train, test])
    out["fit_coef"] = op.model.coef_
    out["solve_y"] = op.solve(ivp).discrete_y()
    np.savez_compressed(os.path.join(HERE, "sml_cases.npz"), **out)
    print("sml_cases: done")


if __name__ == "__main__":
    if sys.argv[1:] == ["solution_interp_diff"]:
        solution_case()
    elif sys.argv[1:] == ["sml_cases"]:
        sml_case()
    else:
        main()
