"""Slice-sharded Parareal driving the fused stencil kernels (needs a GB300).

One rank (no process group): ``SliceShardedParareal`` with
``FDMSlicePropagator`` fine and coarse propagators reproduces the reference's
own multi-rank Parareal output (golden fixtures made by running the
reference's PararealOperator on thread-ranks) to REL_F64 = 1e-12 relative L2,
the same bar as the batched single-GPU operator.
"""

import numpy as np
import pytest

import pararealml_gb300 as ns
from golden_cases import BATCHED_ONLY_PARAREAL, PARAREAL_CASES, load, rel_l2
from pararealml_gb300.operators import fdm
from pararealml_gb300.operators.parareal import FDMSlicePropagator, SliceShardedParareal

pytestmark = pytest.mark.gpu

REL_F64 = 1e-12


def _fdm(integ, d_t):
    return fdm.FDMOperator(getattr(fdm, integ)(), fdm.ThreePointCentralDifferenceMethod(), d_t)


@pytest.mark.parametrize("name", sorted(set(PARAREAL_CASES) - set(BATCHED_ONLY_PARAREAL)))
def test_sharded_parareal_matches_reference_multi_rank_parareal(name):
    import torch

    builder, kw, fi, fdt, gi, gdt, ranks, tol, max_it = PARAREAL_CASES[name]
    gold = load(name)
    ivp = builder(ns, **kw)
    cp = ivp.constrained_problem
    t0, t1 = ivp.t_interval
    delta = (t1 - t0) / ranks
    fine = FDMSlicePropagator(_fdm(fi, fdt), cp, ranks, delta, trajectory=True)
    coarse = FDMSlicePropagator(_fdm(gi, gdt), cp, 1, delta)
    op = SliceShardedParareal(fine, coarse, tol, max_it, fine_trajectory=fine.steps, coarse_whole=coarse.whole)
    y0 = torch.tensor(np.asarray(ivp.initial_condition.discrete_y_0(True), dtype=np.float64), device="cuda")
    out = op.solve(y0, (t0, t1), ranks)
    y = out["trajectory"].cpu().numpy()
    assert y.shape[0] == int(gold["n_steps"])
    assert rel_l2(y[gold["steps"] - 1], gold["y"]) < REL_F64
    assert op.last_stats["world"] == 1
