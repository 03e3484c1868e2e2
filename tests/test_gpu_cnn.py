"""GPU CNN kernels against the CPU oracle (needs a GB300).

The oracle (``oracle/cnn.py``) computes in float64 and rounds to bfloat16
where the GPU stores bfloat16, so the only differences left are float32
accumulation order and the occasional bfloat16 rounding flip that order
causes.  Bars: network output within REL_FWD = 5e-3 relative L2; every
weight and bias gradient within REL_GRAD = 3e-2 relative L2.
"""

import numpy as np
import pytest

from oracle import cnn as ocnn

pytestmark = pytest.mark.gpu

REL_FWD = 5e-3
REL_GRAD = 3e-2


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def _planar(u_nhwc, pitch):
    import torch

    B, H, W, C = u_nhwc.shape
    out = np.zeros((B, C, H, pitch), dtype=np.float32)
    out[..., :W] = np.transpose(u_nhwc, (0, 3, 1, 2))
    return torch.from_numpy(out).cuda()


def _setup(B=2, H=19, W=45, seed=0):
    from pararealml_gb300.learned import ResidualCNN

    rng = np.random.default_rng(seed)
    params = ocnn.init_params(seed)
    for k in params:
        if k.startswith("b"):
            params[k] = rng.normal(0.0, 0.05, params[k].shape)
    u = rng.normal(0.0, 0.5, (B, H, W, 2)).astype(np.float32).astype(np.float64)
    s_in = np.array([1.7, 0.6])
    s_out = np.array([0.05, 0.2])
    model = ResidualCNN(params)
    model.set_scales(s_in.tolist(), s_out.tolist())
    return model, params, u, s_in.astype(np.float32).astype(np.float64), s_out.astype(np.float32).astype(np.float64)


def test_forward_matches_oracle():
    import torch

    model, params, u, s_in, s_out = _setup()
    B, H, W, _ = u.shape
    pitch = 64
    ud = _planar(u, pitch)
    yd = torch.zeros_like(ud)
    model.forward(ud, yd, H, W)
    y = yd[..., :W].permute(0, 2, 3, 1).cpu().numpy().astype(np.float64)
    want, _ = ocnn.forward(params, u, s_in, s_out)
    assert _rel(y - u, want - u) < REL_FWD


def test_gradients_match_oracle():
    import torch

    model, params, u, s_in, s_out = _setup(seed=1)
    B, H, W, _ = u.shape
    pitch = 64
    ud = _planar(u, pitch)
    yd = torch.zeros_like(ud)
    model.forward(ud, yd, H, W)
    rng = np.random.default_rng(5)
    dy = rng.normal(0.0, 1.0, (B, 2, H, W))
    model.backward(ud, H, W, dy=torch.tensor(dy, dtype=torch.float32, device="cuda"))
    got = model.host_grads()
    _, cache = ocnn.forward(params, u, s_in, s_out)
    want = ocnn.backward(params, cache, np.transpose(dy, (0, 2, 3, 1)), s_in, s_out)
    for k in want:
        assert _rel(got[k], want[k]) < REL_GRAD, k


def test_training_reduces_the_loss_on_a_learnable_map():
    """Learn one explicit diffusion step u -> u + 0.1 * lap(u) (zero halo)."""
    import torch

    from pararealml_gb300.learned import CNNCoarseOperator

    rng = np.random.default_rng(2)
    N, H, W, pitch = 64, 24, 40, 64
    u = rng.normal(0.0, 1.0, (N, H, W, 2))
    lap = sum(ocnn.shift(u, dy, dx) for dy, dx in ((1, 0), (-1, 0), (0, 1), (0, -1))) - 4 * u
    v = u + 0.1 * lap
    x = _planar(u, pitch)
    t = _planar(v, pitch)
    op = CNNCoarseOperator(0.05)
    losses = op.train(x, t, H, W, epochs=25, batch=16, lr=3e-3, lr_decay=0.95)
    assert losses[-1] < 0.1 * losses[0]


def test_learned_correction_beats_its_base_coarse_operator():
    """What the trained network gains: on held-out Cahn-Hilliard states the
    CNN-corrected coarse step (forward Euler dt 0.0125 + learned correction)
    is closer to the fine propagator over 0.05 than forward Euler alone, and
    Parareal's first updates are smaller with it."""
    import torch

    import pararealml_gb300 as ns
    import problems
    from pararealml_gb300.learned import CNNCoarseOperator, generate_pairs
    from pararealml_gb300.operators import fdm
    from pararealml_gb300.operators.parareal import PararealOperator

    n, length, t_end = 64, 16.0, 0.8
    fine = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 1e-3, dtype="float32", trajectory="final")
    base = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.0125, dtype="float32")
    train_ivps = [problems.cahn_hilliard_2d(ns, n=n, length=length, t_end=t_end, seed=100 + k) for k in range(32)]
    cp = train_ivps[0].constrained_problem
    y0s = np.stack([ivp.initial_condition.discrete_y_0(True) for ivp in train_ivps])
    x, tgt = generate_pairs(fine, cp, y0s, t_end, 0.05)
    ml = CNNCoarseOperator(0.05, base=base)
    ml.train(x, tgt, n + 1, n + 1, epochs=15, batch=16, lr=2e-3, lr_decay=0.9, cp=cp)

    test_ivps = [problems.cahn_hilliard_2d(ns, n=n, length=length, t_end=t_end, seed=900 + k) for k in range(4)]
    # same constrained problem object for the held-out states
    y0t = np.stack([ivp.initial_condition.discrete_y_0(True) for ivp in test_ivps])
    xt, tt = generate_pairs(fine, cp, y0t, t_end, 0.05)
    prop_ml = ml.coarse_propagator(cp, xt.shape[0], 1)
    y_ml = torch.empty_like(xt)
    prop_ml(xt, y_ml, 0.0)
    y_fe = torch.empty_like(xt)
    ml.apply_base(cp, xt, y_fe)
    e_ml = float(torch.linalg.norm((y_ml - tt)[..., : n + 1]))
    e_fe = float(torch.linalg.norm((y_fe - tt)[..., : n + 1]))
    assert e_ml < 0.7 * e_fe, (e_ml, e_fe)

    ivp = ns.InitialValueProblem(cp, (0.0, t_end), test_ivps[0].initial_condition)
    norms = {}
    for name, g in (("ml", ml), ("fe", fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.0125, dtype="float32"))):
        op = PararealOperator(fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 1e-3, dtype="float32"),
                              g, 1e-12, 2, n_slices=8, trajectory="final")
        op.solve(ivp)
        norms[name] = [float(np.max(h)) for h in op.last_stats["norm_history"]]
    assert norms["ml"][0] < norms["fe"][0]
