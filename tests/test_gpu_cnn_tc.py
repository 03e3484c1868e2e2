"""tcgen05 32 -> 32 convolutions (TMEM accumulators) against a float64
numpy convolution of the same bf16 inputs and against the mma.sync kernel
(needs a GB300).

Both kernels read bf16 inputs exactly and accumulate in float32 in
different orders, then round to bf16, so they may differ by a rounding of
the output.  Bars: relative L2 error against the float64 convolution below
REL = 4e-3 (bf16 output rounding is 2^-9 relative), and the two kernels
within REL of each other.  Shapes: a partial 128-pixel segment, rows of
three segments, a 1-pixel last segment, and enough tiles that every CTA
walks several (both accumulators, every stage of the load ring).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 4e-3


def _bf16(a):
    import torch

    return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16)


def _conv_ref(x, w, bias=None, mask=None):
    """x [B,H,W,32] f64, w [9][n][k] f64: y[p][n] = sum_tap,k w[tap][n][k] x[p+tap][k]."""
    B, H, W, _ = x.shape
    xp = np.zeros((B, H + 2, W + 2, 32))
    xp[:, 1:-1, 1:-1] = x
    y = np.zeros((B, H, W, 32))
    for tap in range(9):
        dy, dx = tap // 3, tap % 3
        y += np.einsum("bhwk,nk->bhwn", xp[:, dy : dy + H, dx : dx + W], w[tap])
    if bias is not None:
        y = np.maximum(y + bias, 0.0)
    if mask is not None:
        y = np.where(mask > 0, y, 0.0)
    return y


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("B,H,W", [(2, 19, 45), (1, 7, 300), (3, 33, 129), (4, 257, 257)])
def test_tcgen05_convolutions_match(B, H, W):
    import torch

    from pararealml_gb300 import _native

    lib = _native.lib()
    rng = np.random.default_rng(B * 1000 + H * 10 + W)
    x = _bf16(rng.normal(0.0, 1.0, (B, H, W, 32))).cuda()
    msk = _bf16(rng.normal(0.0, 1.0, (B, H, W, 32))).cuda()
    w = _bf16(rng.normal(0.0, 0.1, (9, 32, 32))).cuda()
    bias = torch.tensor(rng.normal(0.0, 0.1, 32), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    xf, wf, mf = (t.float().cpu().numpy().astype(np.float64) for t in (x, w, msk))
    want = {0: _conv_ref(xf, wf, bias=bias.cpu().numpy()), 1: _conv_ref(xf, wf, mask=mf)}
    got = {}
    prev = lib.prml_cnn_set_tensor_path(1)
    try:
        for path in (1, 0):
            lib.prml_cnn_set_tensor_path(path)
            y0 = torch.full_like(x, float("nan"))
            y1 = torch.full_like(x, float("nan"))
            _native.check(lib.prml_cnn_mid_fwd(x.data_ptr(), w.data_ptr(), bias.data_ptr(), y0.data_ptr(), B, H, W, s),
                          "mid fwd")
            _native.check(lib.prml_cnn_mid_dgrad(x.data_ptr(), w.data_ptr(), msk.data_ptr(), y1.data_ptr(), B, H, W, s),
                          "mid dgrad")
            torch.cuda.synchronize()
            _native.check(lib.prml_cnn_status(), "tcgen05 status")
            got[path] = (y0.float().cpu().numpy(), y1.float().cpu().numpy())
    finally:
        lib.prml_cnn_set_tensor_path(prev)
    for mode in (0, 1):
        tc, legacy = got[1][mode], got[0][mode]
        assert np.all(np.isfinite(tc)), mode
        assert _rel(tc, want[mode]) < REL, (mode, _rel(tc, want[mode]))
        assert _rel(legacy, want[mode]) < REL, (mode, _rel(legacy, want[mode]))
        assert _rel(tc, legacy) < REL, mode


REL_WG = 1e-4  # float32 accumulation over up to 4 x 257^2 pixels of exact bf16 products


@pytest.mark.parametrize("B,H,W", [(2, 19, 45), (1, 7, 300), (3, 33, 129), (4, 257, 257)])
def test_tcgen05_weight_gradient_matches(B, H, W):
    """dW[tap][ci][co] = sum_p x[p + tap][ci] g[p][co] and db = sum_p g[p]:
    the tcgen05 kernel (K = pixels, both operands read MN-major from the
    staged NHWC rows) and the mma.sync kernel against a float64 sum of the
    same bf16 inputs."""
    import torch

    from pararealml_gb300 import _native

    lib = _native.lib()
    rng = np.random.default_rng(7 * B + H + W)
    x = _bf16(rng.normal(0.0, 1.0, (B, H, W, 32))).cuda()
    g = _bf16(rng.normal(0.0, 1.0, (B, H, W, 32))).cuda()
    parts = 608
    scratch = torch.empty(lib.prml_cnn_wgrad_scratch_elems(parts), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    xf, gf = (t.float().cpu().numpy().astype(np.float64) for t in (x, g))
    xp = np.zeros((B, H + 2, W + 2, 32))
    xp[:, 1:-1, 1:-1] = xf
    want = np.stack([np.einsum("bhwk,bhwn->kn", xp[:, t // 3: t // 3 + H, t % 3: t % 3 + W], gf) for t in range(9)])
    got = {}
    prev = lib.prml_cnn_set_tensor_path(1)
    try:
        for path in (1, 0):
            lib.prml_cnn_set_tensor_path(path)
            dw = torch.full((9, 32, 32), float("nan"), dtype=torch.float32, device="cuda")
            db = torch.full((32,), float("nan"), dtype=torch.float32, device="cuda")
            _native.check(lib.prml_cnn_mid_wgrad(x.data_ptr(), g.data_ptr(), dw.data_ptr(), db.data_ptr(), parts,
                                                 scratch.data_ptr(), B, H, W, s), "mid wgrad")
            torch.cuda.synchronize()
            _native.check(lib.prml_cnn_status(), "tcgen05 status")
            got[path] = (dw.cpu().numpy().astype(np.float64), db.cpu().numpy().astype(np.float64))
    finally:
        lib.prml_cnn_set_tensor_path(prev)
    for path in (1, 0):
        dw, db = got[path]
        assert np.all(np.isfinite(dw)), path
        assert _rel(dw, want) < REL_WG, (path, _rel(dw, want))
        assert _rel(db, gf.sum(axis=(0, 1, 2))) < REL_WG, path
    assert _rel(got[1][0], got[0][0]) < REL_WG
