"""Parity at the benchmark configurations' own sizes (needs a GB300).

The golden fixtures pin the GPU path on small meshes; these tests run the
configured workloads at their full mesh sizes against the CPU oracle (the
numpy restatement of the reference) on shortened time spans, and the
batched Parareal configuration in full against its float64 serial solve.

* 2D Cahn-Hilliard at 1025^2 (the benchmark's default workload), RK4
  dt 1e-4: float64 within 1e-12 relative L2 of the oracle after 10 steps in
  both operation orders; float32 and compensated float32 at their stated
  bars.
* The uneven-size shallow-water ensemble: one instance of each mesh size
  (65^2, 129^2, 257^2, 513^2) through the ensemble solver, RK4 at CFL 0.4
  to t = 0.1 (7 / 4 / 2 / 1 steps), float64 within 1e-12 of the oracle.
* Batched Parareal on 2D diffusion at 257^2, t in [0, 4], 32 slices, fine
  RK4 1e-4, coarse forward Euler 2.5e-4, tol 1e-6 (8 of the 64 seeded
  Gaussian initial conditions): float64 solvers reach the float64 serial
  solve within 1e-6 relative L2.  Float32 stencils cannot: a second
  difference of a smooth field rounded to 24 bits carries a relative error
  of about u / (k dx)^2 (u = 6e-8, k dx ~ 0.05 for these Gaussians), so
  every float32 right-hand side is off by ~1e-4 relative, and the
  compensated state (which keeps the rounding of each increment, not of the
  right-hand side) ends the 40,000 steps at ~6e-5; their bar is 2e-4.
"""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import rel_l2
from oracle import fdm as orc
from pararealml_gb300.operators import fdm

pytestmark = pytest.mark.gpu

REL_F64 = 1e-12


def _rk4(d_t, **kw):
    return fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), d_t, **kw)


@pytest.fixture(scope="module")
def cahn_hilliard_1025():
    """The default benchmark workload's problem and 10 oracle RK4 steps."""
    ivp = problems.cahn_hilliard_2d(ns, n=1024, length=64.0, t_end=10 * 1e-4, seed=541016860)
    y0 = ivp.initial_condition.discrete_y_0(True)
    st = orc.FDMStepper(ivp.constrained_problem, orc.RK4, 1e-4)
    y = np.array(y0)
    for i in range(10):
        y = st.step(i * 1e-4, y)
    return ivp, y


@pytest.mark.parametrize("op_order", ["fused", "reference"])
def test_cahn_hilliard_1025_float64_matches_oracle(cahn_hilliard_1025, op_order):
    ivp, want = cahn_hilliard_1025
    got = _rk4(1e-4, trajectory="final", op_order=op_order).solve(ivp).discrete_y()[-1]
    err = rel_l2(got, want)
    print(f"1025^2 Cahn-Hilliard float64 ({op_order}) rel L2 after 10 steps: {err:.3e}")
    assert err < REL_F64


@pytest.mark.parametrize("dtype,bar", [("float32", 1e-5), ("float32c", 1e-6)])
def test_cahn_hilliard_1025_float32_bars(cahn_hilliard_1025, dtype, bar):
    """Float32 rounds the state (c and the LHS.Y row mu) to 24 bits every
    step; the compensated state carries the rounding of c's increments, and
    mu, recomputed from c each step, keeps float32 resolution."""
    ivp, want = cahn_hilliard_1025
    got = _rk4(1e-4, trajectory="final", dtype=dtype).solve(ivp).discrete_y()[-1]
    err = rel_l2(got, want)
    err_c = rel_l2(got[..., 0], want[..., 0])
    print(f"1025^2 Cahn-Hilliard {dtype} rel L2 after 10 steps: {err:.3e} (c alone {err_c:.3e})")
    assert err < bar


def test_shallow_water_ensemble_each_size_matches_oracle():
    from pararealml_gb300.ensemble import EnsembleSolver

    ivps, d_ts = problems.shallow_water_ensemble(ns, n_instances=64, t_end=0.1)
    picked = {}
    for ivp, d_t in zip(ivps, d_ts):
        n = ivp.constrained_problem.mesh.vertices_shape[0]
        picked.setdefault(n, (ivp, d_t))
    assert sorted(picked) == [65, 129, 257, 513]
    sel = [picked[n] for n in sorted(picked)]
    for dtype, bar in (("float64", REL_F64), ("float32", 1e-5)):
        solver = EnsembleSolver(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), dtype=dtype)
        solver.setup([s[0] for s in sel], [s[1] for s in sel])
        solver.advance()
        got = solver.final_states()
        for (ivp, d_t), y in zip(sel, got):
            y0 = ivp.initial_condition.discrete_y_0(True)
            want = orc.fdm_solve(ivp.constrained_problem, y0, ivp.t_interval, d_t, orc.RK4, keep="final")
            err = rel_l2(y, want)
            print(f"shallow water {y.shape[0]}^2 {dtype} ({int(round(0.1 / d_t))} steps): rel L2 {err:.3e}")
            assert err < bar


def test_batched_parareal_diffusion_257_reaches_1e6():
    from pararealml_gb300.operators.parareal import PararealOperator

    n, slices, t_end, n_ic = 256, 32, 4.0, 8
    rng = np.random.default_rng(problems.SEEDS[1])
    means = rng.uniform(2.0, 8.0, (64, 2))[:n_ic]
    scales = rng.uniform(0.3, 1.0, 64)[:n_ic]
    mesh = ns.Mesh([(0.0, 10.0), (0.0, 10.0)], [10.0 / n, 10.0 / n])
    bc = ns.DirichletBoundaryCondition(lambda x, t: np.zeros((len(x), 1)), is_static=True)
    cp = ns.ConstrainedProblem(ns.DiffusionEquation(2), mesh, [(bc, bc)] * 2)
    y0 = np.stack([ns.GaussianInitialCondition(cp, [(means[k], scales[k] * np.eye(2))],
                                               [2.0 * np.pi * scales[k]]).discrete_y_0(True) for k in range(n_ic)])
    n_steps = int(round(t_end / 1e-4))

    def serial(dtype):
        op = _rk4(1e-4, dtype=dtype, trajectory="final")
        plan = op.plan(cp, n_ic)
        s0 = plan.new_state(1)
        plan.pack(y0, s0[0])
        end = plan.new_state(1)
        plan.run(s0[0], end, n_steps, 0.0, 1e-4, n_steps)
        return plan.unpack(end[0], n_ic).cpu().numpy()

    ref = serial("float64")
    err32 = rel_l2(serial("float32"), ref)
    err32c = rel_l2(serial("float32c"), ref)

    def parareal(dtype):
        fine = _rk4(1e-4, dtype=dtype, trajectory="final")
        coarse = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 2.5e-4,
                                 dtype=dtype)
        op = PararealOperator(fine, coarse, 1e-6, n_slices=slices, trajectory="final")
        res = op.run(cp, y0, (0.0, t_end))
        errs = [rel_l2(res["final"][k].cpu().numpy(), ref[k]) for k in range(n_ic)]
        return max(errs), np.asarray(op.last_stats["iterations"]).reshape(-1).tolist()

    e64, it64 = parareal("float64")
    e32c, it32c = parareal("float32c")
    print(f"batched Parareal, diffusion 257^2 (8 ICs): serial float32 {err32:.3e}, float32c {err32c:.3e}; Parareal float64 {e64:.3e} "
          f"(iterations {it64}), float32c {e32c:.3e} (iterations {it32c})")
    assert e64 < 1e-6
    assert err32 < 2e-4 and err32c < 2e-4 and e32c < 2e-4
