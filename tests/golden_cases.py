"""Golden fixture catalogue shared by the CPU oracle tests and the GPU tests."""

from __future__ import annotations

import os

import numpy as np

import problems

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# name -> (builder, kwargs, integrator name, d_t)
FDM_CASES = {
    "diffusion_fe_65": (problems.diffusion_2d, dict(n=64, t_end=2.0), "ForwardEulerMethod", 0.0025),
    "diffusion_rk4": (problems.diffusion_2d, dict(n=32, t_end=0.5), "RK4", 0.01),
    "diffusion_midpoint": (problems.diffusion_2d, dict(n=32, t_end=0.5), "ExplicitMidpointMethod", 0.01),
    "cahn_hilliard_rk4": (problems.cahn_hilliard_2d, dict(n=32, length=8.0, t_end=0.05), "RK4", 0.001),
    "cahn_hilliard_fe": (problems.cahn_hilliard_2d, dict(n=32, length=8.0, t_end=0.05), "ForwardEulerMethod", 0.001),
    "shallow_water_rk4": (problems.shallow_water_2d, dict(n=32, length=64.0, t_end=2.0), "RK4", 0.1),
    "wave_mixed_rk4": (problems.mixed_bc_wave_2d, dict(nx=24, ny=20, t_end=0.1), "RK4", 0.005),
    "wave_mixed_midpoint": (problems.mixed_bc_wave_2d, dict(nx=24, ny=20, t_end=0.1), "ExplicitMidpointMethod", 0.005),
    "burgers_rk4": (problems.burgers_2d, dict(n=24, t_end=0.05), "RK4", 0.001),
    "convdiff_1d_fe": (problems.convection_diffusion_1d, dict(n=50, t_end=0.2), "ForwardEulerMethod", 0.01),
    "population_growth_rk4": (problems.population_growth, dict(t_end=1.0), "RK4", 0.01),
    "diffusion_1d_dynamic_rk4": (problems.dynamic_bc_diffusion_1d, dict(), "RK4", 0.5),
    "wave_dynamic_rk4": (problems.dynamic_bc_wave_2d, dict(), "RK4", 0.002),
    "wave_dynamic_fe": (problems.dynamic_bc_wave_2d, dict(), "ForwardEulerMethod", 0.001),
    "wave_dynamic_midpoint": (problems.dynamic_bc_wave_2d, dict(), "ExplicitMidpointMethod", 0.002),
    "cahn_hilliard_3d_rk4": (problems.cahn_hilliard_3d, dict(), "RK4", 0.05),
    "diffusion_3d_rk4": (problems.diffusion_3d_mixed, dict(), "RK4", 0.001),
    "diffusion_3d_fe": (problems.diffusion_3d_mixed, dict(), "ForwardEulerMethod", 0.0005),
    "polar_shallow_water_rk4": (problems.polar_shallow_water, dict(), "RK4", 0.1),
    "cylindrical_diffusion_rk4": (problems.curvilinear_diffusion_3d, dict(system="CYLINDRICAL"), "RK4", 0.1),
    "spherical_diffusion_rk4": (problems.curvilinear_diffusion_3d, dict(system="SPHERICAL"), "RK4", 0.1),
    "spherical_vector_rk4": (problems.curvilinear_vector_field, dict(system="SPHERICAL"), "RK4", 0.001),
    "cylindrical_vector_fe": (problems.curvilinear_vector_field, dict(system="CYLINDRICAL"), "ForwardEulerMethod", 0.0005),
    "navier_stokes_rk4": (problems.navier_stokes_2d, dict(), "RK4", 0.25),
    "jacobi_cartesian_1d_rk4": (problems.jacobi_system, dict(system="CARTESIAN", dims=1), "RK4", 0.005),
    "jacobi_cartesian_2d_rk4": (problems.jacobi_system, dict(system="CARTESIAN", dims=2), "RK4", 0.005),
    "jacobi_cartesian_3d_rk4": (problems.jacobi_system, dict(system="CARTESIAN", dims=3), "RK4", 0.005),
    "jacobi_polar_rk4": (problems.jacobi_system, dict(system="POLAR", dims=2), "RK4", 0.005),
    "jacobi_cylindrical_rk4": (problems.jacobi_system, dict(system="CYLINDRICAL", dims=3), "RK4", 0.005),
    "jacobi_spherical_rk4": (problems.jacobi_system, dict(system="SPHERICAL", dims=3), "RK4", 0.005),
    "jacobi_dynamic_fe": (problems.jacobi_system, dict(system="CARTESIAN", dims=2, dynamic=True), "ForwardEulerMethod", 0.005),
    "diffusion_be": (problems.diffusion_2d, dict(n=32, t_end=0.1), "BackwardEulerMethod", 0.01),
    "cahn_hilliard_cn": (problems.cahn_hilliard_2d, dict(n=32, length=8.0, t_end=0.01), "CrankNicolsonMethod", 0.001),
    "cahn_hilliard_cn07": (problems.cahn_hilliard_2d, dict(n=32, length=8.0, t_end=0.01), "CrankNicolsonMethod:0.7", 0.001),
    "wave_dynamic_be": (problems.dynamic_bc_wave_2d, dict(), "BackwardEulerMethod", 0.002),
    "convdiff_1d_cn": (problems.convection_diffusion_1d, dict(n=50, t_end=0.2), "CrankNicolsonMethod", 0.01),
    "diffusion_3d_be": (problems.diffusion_3d_mixed, dict(), "BackwardEulerMethod", 0.002),
    "navier_stokes_cn": (problems.navier_stokes_2d, dict(t_end=2.0), "CrankNicolsonMethod", 0.25),
}

PARAREAL_CASES = {
    "parareal_diffusion": (problems.diffusion_2d, dict(n=32, t_end=1.0), "RK4", 0.005, "ForwardEulerMethod", 0.0125, 4, 1e-6, 100),
    "parareal_cahn_hilliard_maxit": (problems.cahn_hilliard_2d, dict(n=24, length=6.0, t_end=0.08), "RK4", 0.001, "ForwardEulerMethod", 0.004, 4, 1e-9, 2),
    "parareal_dynamic_diffusion_1d": (problems.dynamic_bc_diffusion_1d, dict(), "RK4", 0.1, "ForwardEulerMethod", 0.25, 4, 1e-6, 100),
    "parareal_dynamic_wave": (problems.dynamic_bc_wave_2d, dict(t_end=0.04), "RK4", 0.001, "ForwardEulerMethod", 0.0025, 4, 1e-6, 100),
    "parareal_implicit_diffusion": (problems.diffusion_2d, dict(n=16, t_end=0.2), "CrankNicolsonMethod", 0.01, "BackwardEulerMethod", 0.05, 4, 1e-6, 100),
}
# cases the batched Parareal takes and the slice-sharded runner does not
# (time-dependent boundary conditions, implicit operators)
BATCHED_ONLY_PARAREAL = ("parareal_dynamic_diffusion_1d", "parareal_dynamic_wave", "parareal_implicit_diffusion")

ORACLE_INTEGRATOR = {"ForwardEulerMethod": "fe", "ExplicitMidpointMethod": "midpoint", "RK4": "rk4",
                     "BackwardEulerMethod": "be", "CrankNicolsonMethod": "cn"}
IMPLICIT_NAMES = ("BackwardEulerMethod", "CrankNicolsonMethod")


def integrator_spec(integ: str):
    """("CrankNicolsonMethod", [0.7]) from "CrankNicolsonMethod:0.7"."""
    name, _, args = integ.partition(":")
    return name, [float(v) for v in args.split(",") if v]


def make_integrator(module, integ: str):
    """The integrator object of a case from ``module`` (this package's fdm
    operators or the reference's)."""
    name, args = integrator_spec(integ)
    return getattr(module, name)(*args)


def oracle_integrator(integ: str):
    """(oracle kind, FDMStepper keyword arguments) of a case's integrator."""
    name, args = integrator_spec(integ)
    kw = {"cn_a": args[0]} if (name == "CrankNicolsonMethod" and args) else {}
    return ORACLE_INTEGRATOR[name], kw


def is_implicit(integ: str) -> bool:
    return integrator_spec(integ)[0] in IMPLICIT_NAMES


def load(name: str):
    return np.load(os.path.join(GOLDEN_DIR, f"{name}.npz"))


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
