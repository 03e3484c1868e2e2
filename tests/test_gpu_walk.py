"""GPU parity of the register-window step kernels (``walk_body``).

Single-stage steps (forward Euler, and stage-invariant systems such as
Cahn-Hilliard under RK4) on 2D meshes have a second kernel family that reads
each thread's window of the state straight into registers instead of staging
tiles in shared memory.  Both families evaluate the same generated
right-hand sides through the same ``Point`` operators, so in float64 their
results are identical bit for bit; against the reference's goldens the bars
are those of the staged kernels (float64 1e-12, float32 5e-5 relative L2).
"""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import FDM_CASES, load, rel_l2
from pararealml_gb300 import codegen
from pararealml_gb300.operators import fdm

pytestmark = pytest.mark.gpu

REL_F64 = 1e-12
REL_F32 = 5e-5
STAGED = (16, 32, 128)


def _op(integ, d_t, **kw):
    return fdm.FDMOperator(getattr(fdm, integ)(), fdm.ThreePointCentralDifferenceMethod(), d_t, **kw)


def _walk(rw, dtype):
    return codegen.walk_tile(rw[0], rw[1], 8 if dtype == "float64" else 4)


@pytest.mark.parametrize("max_ctas", [0, 3])
@pytest.mark.parametrize("rw", list(codegen.WALK_CONFIGS))
@pytest.mark.parametrize("name", ["cahn_hilliard_rk4", "cahn_hilliard_fe", "diffusion_fe_65", "wave_dynamic_fe",
                                  "jacobi_dynamic_fe"])
def test_every_register_window_shape(name, rw, max_ctas):
    """Every register-window shape against the reference's goldens; with
    max_ctas = 3 each CTA walks many tiles."""
    builder, kw, integ, d_t = FDM_CASES[name]
    gold = load(name)
    ivp = builder(ns, **kw)
    for dtype, tol in (("float64", REL_F64), ("float32", REL_F32)):
        np.random.seed(problems.JACOBI_SEED)
        op = _op(integ, d_t, tile=_walk(rw, dtype), max_ctas=max_ctas, dtype=dtype)
        y = op.solve(ivp).discrete_y()
        assert op.plan(ivp.constrained_problem, 1).last_tile == _walk(rw, dtype)
        assert rel_l2(y[gold["steps"] - 1], gold["y"]) < tol, dtype


def _forward_euler_cases():
    return [
        ("cahn_hilliard_ragged", problems.cahn_hilliard_2d(ns, n=131, length=32.75, t_end=0.012), 0.001),
        ("wave_partial_faces", problems.mixed_bc_wave_2d(ns, nx=77, ny=45, t_end=0.012), 0.001),
        ("wave_dynamic_faces", problems.dynamic_bc_wave_2d(ns, nx=26, ny=21, t_end=0.012), 0.001),
        ("diffusion_small", problems.diffusion_2d(ns, n=4, t_end=0.012), 0.001),
    ]


@pytest.mark.parametrize("case", range(4))
@pytest.mark.parametrize("rw", [(1, 4), (2, 4), (4, 2)])
def test_register_window_equals_the_staged_kernel_bit_for_bit(case, rw):
    """Forward Euler on ragged meshes with Neumann faces, partially
    NaN-masked Dirichlet / Neumann faces and time-dependent faces, and a
    5 x 5 mesh (every warp at a face): float64 results identical to the
    staged kernel's, for full trajectories, strided saves and final
    states."""
    _, ivp, d_t = _forward_euler_cases()[case]
    for trajectory in ("full", 2, "final"):
        want = _op("ForwardEulerMethod", d_t, tile=STAGED, trajectory=trajectory).solve(ivp).discrete_y()
        got = _op("ForwardEulerMethod", d_t, tile=_walk(rw, "float64"), trajectory=trajectory).solve(ivp).discrete_y()
        assert np.array_equal(got, want), (trajectory, float(np.max(np.abs(got - want))))


def test_register_window_batches_and_compensated_state():
    """A batch of Cahn-Hilliard instances (RK4, stage-invariant) through
    the device-level solve: each instance equals its staged-kernel result in
    float64; in compensated float32 the window kernel reads every
    instance's own rounding remainders (results within 1e-7 of the staged
    kernel's and of float64)."""
    import torch

    ivps = [problems.cahn_hilliard_2d(ns, n=70, length=17.5, seed=s) for s in (1, 2, 3)]
    cp = ivps[0].constrained_problem
    y0 = torch.tensor(np.stack([ivp.initial_condition.discrete_y_0(True) for ivp in ivps]), device="cuda")
    out = {}
    for dtype in ("float64", "float32c"):
        for name, tile in (("walk", _walk((2, 4), dtype)), ("staged", STAGED)):
            op = _op("RK4", 0.001, tile=tile, dtype=dtype)
            plan = op.plan(cp, 3)
            traj = op.solve_device(cp, y0, 0.0, 12)
            out[dtype, name] = plan.unpack(traj, 12 * 3).cpu().numpy().reshape((12, 3) + tuple(y0.shape[1:]))
    assert np.array_equal(out["float64", "walk"], out["float64", "staged"])
    for b in range(3):
        ref = out["float64", "staged"][:, b]
        assert rel_l2(out["float32c", "walk"][:, b], out["float32c", "staged"][:, b]) < 1e-7
        assert rel_l2(out["float32c", "walk"][:, b], ref) < 1e-7


def test_autotuner_may_pick_either_family():
    """The register-window shapes are candidates of the tile autotuner for
    single-stage 2D steps and absent otherwise (multi-stage RK4, 1D, 3D)."""
    low2 = codegen.lower_problem(problems.cahn_hilliard_2d(ns, n=16).constrained_problem)
    gen = codegen.generate_source(low2, codegen.RK4, "f64", fast=True)
    assert any(codegen.is_walk(t) for t in gen.step_kernels)
    low_sw = codegen.lower_problem(problems.shallow_water_2d(ns, n=16).constrained_problem)
    assert not any(codegen.is_walk(t) for t in codegen.generate_source(low_sw, codegen.RK4, "f64").step_kernels)
    low1 = codegen.lower_problem(problems.convection_diffusion_1d(ns, n=20).constrained_problem)
    assert not any(codegen.is_walk(t) for t in
                   codegen.generate_source(low1, codegen.FORWARD_EULER, "f64").step_kernels)
