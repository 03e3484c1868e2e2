"""Gaussian initial states evaluated on the device (needs a GB300).

``gaussian_initial_states`` against the host ``GaussianInitialCondition``
(the reference's evaluation, pararealml/initial_condition.py:150-307:
scipy's multivariate normal density at the Cartesian images of the
vertices, times the multipliers, Dirichlet vertex constraints applied) on
Cartesian 1D/2D/3D and polar meshes, batched: equal within 1e-14 relative
(the device and host ``exp`` may differ in the last bit).
"""

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from golden_cases import rel_l2
from pararealml_gb300.initial_condition import gaussian_initial_states

pytestmark = pytest.mark.gpu


def _check(ivps):
    cp = ivps[0].constrained_problem
    ics = [ivp.initial_condition for ivp in ivps]
    got = gaussian_initial_states(cp, [ic._means_and_covs for ic in ics], [ic._multipliers for ic in ics]).cpu().numpy()
    for b, ic in enumerate(ics):
        want = ic.discrete_y_0(True)
        assert got[b].shape == want.shape
        assert rel_l2(got[b], want) < 1e-14


def test_batched_gaussians_on_a_dirichlet_square():
    rng = np.random.default_rng(problems.SEEDS[1])
    mesh = ns.Mesh([(0.0, 10.0), (0.0, 10.0)], [10.0 / 64, 10.0 / 64])
    bc = ns.DirichletBoundaryCondition(lambda x, t: np.zeros((len(x), 1)), is_static=True)
    cp = ns.ConstrainedProblem(ns.DiffusionEquation(2), mesh, [(bc, bc)] * 2)
    ivps = []
    for _ in range(6):
        mean, s = rng.uniform(2.0, 8.0, 2), rng.uniform(0.3, 1.0)
        ic = ns.GaussianInitialCondition(cp, [(mean, s * np.eye(2))], [2.0 * np.pi * s])
        ivps.append(ns.InitialValueProblem(cp, (0.0, 1.0), ic))
    _check(ivps)


def test_shallow_water_three_components():
    ivps, _ = problems.shallow_water_ensemble(ns, n_instances=12, sizes=(64,), t_end=0.1)
    _check(ivps)


def test_one_and_three_dimensional_and_polar_meshes():
    _check([problems.dynamic_bc_diffusion_1d(ns)])
    _check([problems.diffusion_3d_mixed(ns)])
    _check([problems.polar_shallow_water(ns)])


def test_rejects_mismatched_arguments():
    cp = problems.diffusion_2d(ns, n=8).constrained_problem
    with pytest.raises(ValueError):
        gaussian_initial_states(cp, [[(np.zeros(3), np.eye(3))]])
    with pytest.raises(ValueError):
        gaussian_initial_states(cp, [[(np.zeros(2), np.eye(2))]], [[1.0, 2.0]])
