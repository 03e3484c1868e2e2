"""Learned coarse propagator: a residual CNN trained on FDM fine trajectories.

The reference's ``SupervisedMLOperator``
(``pararealml/operators/ml/supervised/supervised_ml_operator.py:16-357``) is
an ``Operator`` with its own ``d_t`` whose model is trained on trajectories of
an oracle solver and applied autoregressively by ``solve``.  This module keeps
that contract (``CNNCoarseOperator(d_t).train(...)``, ``.solve(ivp)``) with a
GB300 model: a 3x3 convolutional residual network
``u(t + d_t) = u(t) + s_out * net(s_in * u(t))`` (2 -> 32 -> 32 x4 -> 2
channels, ReLU), whose forward, backward and Adam kernels are this package's
own (``csrc/prml_cnn.cu``, BF16 tensor-core implicit GEMM with FP32
accumulation for the 32 -> 32 layers).  Training data come from the GPU FDM
fine solver itself.  As the coarse operator of ``PararealOperator`` it
provides ``coarse_propagator`` (batched device-to-device propagation).
"""

from __future__ import annotations

from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _native
from .operator import Operator, discretize_time_domain
from .solution import Solution

HC = 32
N_MID = 4
LAYERS = N_MID + 2
_SHAPES = [(9, 2, HC)] + [(9, HC, HC)] * N_MID + [(9, HC, 2)]


def _layout():
    off = 0
    out = []
    for l, shp in enumerate(_SHAPES):
        n = int(np.prod(shp))
        out.append(("w", l, off, shp))
        off += n
        out.append(("b", l, off, (shp[-1],)))
        off += shp[-1]
    return out, off


LAYOUT, N_PARAMS = _layout()


def init_params(seed: int = 0) -> Dict[str, np.ndarray]:
    """He-normal weights (last layer scaled by 0.1), zero biases."""
    rng = np.random.default_rng(seed)
    p = {}
    for l, shp in enumerate(_SHAPES):
        scale = np.sqrt(2.0 / (9 * shp[1]))
        if l == LAYERS - 1:
            scale *= 0.1
        p[f"w{l}"] = rng.normal(0.0, scale, shp)
        p[f"b{l}"] = np.zeros(shp[-1])
    return p


class ResidualCNN:
    """Device parameters, optimiser state and workspaces of the network."""

    def __init__(self, params: Optional[Dict[str, np.ndarray]] = None, seed: int = 0, device=None):
        import torch

        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        p = params if params is not None else init_params(seed)
        flat = np.zeros(N_PARAMS, dtype=np.float32)
        for kind, l, off, shp in LAYOUT:
            flat[off: off + int(np.prod(shp))] = np.asarray(p[f"{kind}{l}"], dtype=np.float32).ravel()
        self.params = torch.tensor(flat, device=self.device)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        self.s_in = torch.ones(2, dtype=torch.float32, device=self.device)
        self.s_out = torch.ones(2, dtype=torch.float32, device=self.device)
        self.wf = torch.empty((N_MID, 9 * HC * HC), dtype=torch.bfloat16, device=self.device)
        self.wd = torch.empty_like(self.wf)
        self._work: Dict[tuple, dict] = {}
        self.pack()

    # ---- parameter views
    def _view(self, t, kind, l):
        for k, ll, off, shp in LAYOUT:
            if k == kind and ll == l:
                return t[off: off + int(np.prod(shp))]
        raise KeyError((kind, l))

    def w(self, l, t=None):
        return self._view(self.params if t is None else t, "w", l)

    def b(self, l, t=None):
        return self._view(self.params if t is None else t, "b", l)

    def host_params(self) -> Dict[str, np.ndarray]:
        flat = self.params.cpu().numpy().astype(np.float64)
        out = {}
        for kind, l, off, shp in LAYOUT:
            out[f"{kind}{l}"] = flat[off: off + int(np.prod(shp))].reshape(shp)
        return out

    def host_grads(self) -> Dict[str, np.ndarray]:
        flat = self.grads.cpu().numpy().astype(np.float64)
        return {f"{k}{l}": flat[o: o + int(np.prod(s))].reshape(s) for k, l, o, s in LAYOUT}

    def set_scales(self, s_in: Sequence[float], s_out: Sequence[float]) -> None:
        import torch

        self.s_in.copy_(torch.tensor(s_in, dtype=torch.float32))
        self.s_out.copy_(torch.tensor(s_out, dtype=torch.float32))

    def pack(self) -> None:
        lib = _native.lib()
        for i in range(N_MID):
            _native.check(
                lib.prml_cnn_pack_mid(self.w(i + 1).data_ptr(), self.wf[i].data_ptr(), self.wd[i].data_ptr(), _stream()),
                "pack",
            )

    # ---- workspaces per (batch, H, W)
    def _ws(self, B, H, W):
        import torch

        key = (B, H, W)
        ws = self._work.get(key)
        if ws is None:
            acts = torch.empty((LAYERS - 1, B, H, W, HC), dtype=torch.bfloat16, device=self.device)
            ws = {"acts": acts}
            # kept for the model's lifetime: recorded CUDA graphs may refer to it
            self._work[key] = ws
        return ws

    def _grad_ws(self, ws, B, H, W):
        import torch

        if "g" not in ws:
            lib = _native.lib()
            parts = 608
            ws["g"] = torch.empty((2, B, H, W, HC), dtype=torch.bfloat16, device=self.device)
            ws["dy"] = torch.empty((B, 2, H, W), dtype=torch.float32, device=self.device)
            n = max(lib.prml_cnn_wgrad_scratch_elems(parts), lib.prml_cnn_thin_scratch_elems(parts))
            ws["scratch"] = torch.empty(n, dtype=torch.float32, device=self.device)
            ws["loss_parts"] = torch.empty(parts, dtype=torch.float64, device=self.device)
            ws["parts"] = parts
        return ws

    # ---- forward / backward on planar states (B, 2, H, pitch)
    def forward(self, u, y, H: int, W: int, residual=None) -> None:
        """y = r + s_out * net(s_in * u) with r = ``residual`` (default u);
        u, y, r planar device states (B, 2, H, pitch)."""
        lib = _native.lib()
        B, pitch, es = u.shape[0], u.shape[-1], u.element_size()
        ws = self._ws(B, H, W)
        acts = ws["acts"]
        s = _stream()
        chk = _native.check
        chk(lib.prml_cnn_in_fwd(u.data_ptr(), es, pitch, self.w(0).data_ptr(), self.b(0).data_ptr(),
                                self.s_in.data_ptr(), acts[0].data_ptr(), B, H, W, s), "cnn in")
        for i in range(N_MID):
            chk(lib.prml_cnn_mid_fwd(acts[i].data_ptr(), self.wf[i].data_ptr(), self.b(i + 1).data_ptr(),
                                     acts[i + 1].data_ptr(), B, H, W, s), "cnn mid")
        chk(lib.prml_cnn_out_fwd(acts[N_MID].data_ptr(), self.w(LAYERS - 1).data_ptr(), self.b(LAYERS - 1).data_ptr(),
                                 self.s_out.data_ptr(), (u if residual is None else residual).data_ptr(), y.data_ptr(),
                                 es, pitch, B, H, W, s), "cnn out")

    def loss_and_dy(self, y, target, H: int, W: int) -> "torch.Tensor":
        """Writes dL/dy of the mean squared error into the workspace; returns the loss (device scalar)."""
        lib = _native.lib()
        B, pitch, es = y.shape[0], y.shape[-1], y.element_size()
        ws = self._grad_ws(self._ws(B, H, W), B, H, W)
        _native.check(lib.prml_cnn_mse(y.data_ptr(), target.data_ptr(), es, pitch, B, H, W, ws["dy"].data_ptr(),
                                       ws["loss_parts"].data_ptr(), ws["parts"], _stream()), "mse")
        return ws["loss_parts"].sum() / (B * 2 * H * W)

    def backward(self, u, H: int, W: int, dy=None) -> None:
        """Gradients of the loss (dL/dy in the workspace, or ``dy``) into ``self.grads``."""
        lib = _native.lib()
        B, pitch, es = u.shape[0], u.shape[-1], u.element_size()
        ws = self._grad_ws(self._ws(B, H, W), B, H, W)
        if dy is not None:
            ws["dy"].copy_(dy)
        acts, g, sc, parts, s = ws["acts"], ws["g"], ws["scratch"], ws["parts"], _stream()
        chk = _native.check
        last = LAYERS - 1
        chk(lib.prml_cnn_out_bwd(ws["dy"].data_ptr(), acts[N_MID].data_ptr(), self.w(last).data_ptr(),
                                 self.s_out.data_ptr(), g[0].data_ptr(), self.w(last, self.grads).data_ptr(),
                                 self.b(last, self.grads).data_ptr(), parts, sc.data_ptr(), B, H, W, s), "cnn out bwd")
        cur = 0
        for i in range(N_MID - 1, -1, -1):  # layer i+1 maps acts[i] -> acts[i+1]; g[cur] = dL/d acts[i+1]
            chk(lib.prml_cnn_mid_wgrad(acts[i].data_ptr(), g[cur].data_ptr(), self.w(i + 1, self.grads).data_ptr(),
                                       self.b(i + 1, self.grads).data_ptr(), parts, sc.data_ptr(), B, H, W, s),
                "cnn wgrad")
            chk(lib.prml_cnn_mid_dgrad(g[cur].data_ptr(), self.wd[i].data_ptr(), acts[i].data_ptr(),
                                       g[1 - cur].data_ptr(), B, H, W, s), "cnn dgrad")
            cur = 1 - cur
        chk(lib.prml_cnn_in_wgrad(g[cur].data_ptr(), u.data_ptr(), es, pitch, self.s_in.data_ptr(),
                                  self.w(0, self.grads).data_ptr(), self.b(0, self.grads).data_ptr(), parts,
                                  sc.data_ptr(), B, H, W, s), "cnn in wgrad")

    def adam_step(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        self.step += 1
        _native.check(
            _native.lib().prml_cnn_adam(self.params.data_ptr(), self.grads.data_ptr(), self.m.data_ptr(),
                                        self.v.data_ptr(), N_PARAMS, lr, beta1, beta2, eps, self.step, _stream()),
            "adam",
        )
        self.pack()


def _stream() -> int:
    import torch

    return torch.cuda.current_stream().cuda_stream


def generate_pairs(fine, cp, y0s: np.ndarray, t_end: float, d_t: float):
    """Training pairs (u(t), u(t + d_t)) from batched fine-solver trajectories.

    GPU counterpart of ``SupervisedMLOperator.generate_data``
    (``supervised_ml_operator.py:130-236``): every initial state in ``y0s``
    (float64, (N, *vertices, C)) is advanced by the fine ``FDMOperator`` from
    0 to ``t_end`` in one batched device run that keeps every d_t-th state.
    Returns (inputs, targets) as device states (N * t_end/d_t, C, nx, pitch)
    in the fine operator's precision.
    """
    import torch

    n_out = int(round(t_end / d_t))
    per = int(round(d_t / fine.d_t))
    if not np.isclose(per * fine.d_t, d_t) or not np.isclose(n_out * d_t, t_end):
        raise ValueError("d_t must be a multiple of the fine step and divide t_end")
    n = y0s.shape[0]
    plan = fine.plan(cp, n)
    states = plan.new_state(n_out + 1)
    plan.pack_device(torch.from_numpy(np.ascontiguousarray(y0s, dtype=np.float64)).to(plan.device), states[0])
    plan.run(states[0], states[1:], n_out * per, 0.0, fine.d_t, save_every=per)
    plan.check_status()
    shape = tuple(states.shape[2:])
    inputs = states[:-1].reshape((n_out * n,) + shape)
    targets = states[1:].reshape((n_out * n,) + shape)
    return inputs, targets


class CNNCoarseOperator(Operator):
    """Operator with its own ``d_t`` that advances a 2-component state by the
    trained residual CNN (the reference's ``SupervisedMLOperator`` contract).

    With ``base`` (a cheap, stable coarse ``FDMOperator`` whose step divides
    ``d_t``) the network learns a correction to it:
    ``u(t + d_t) = base(u(t)) + s_out * net(s_in * u(t))``; without it the
    residual is u(t) itself.
    """

    def __init__(self, d_t: float, model: Optional[ResidualCNN] = None, *, base=None, dtype: str = "float32"):
        super().__init__(d_t, True)
        self.model = model
        self.base = base
        self.dtype = "f32" if dtype in ("float32", "f32") else "f64"
        if base is not None:
            n = int(round(d_t / base.d_t))
            if not np.isclose(n * base.d_t, d_t):
                raise ValueError("the base operator's time step must divide d_t")
            if base.dtype != self.dtype:
                raise ValueError("the base operator must use the network's precision")
        self.history: List[float] = []

    def _base_steps(self) -> int:
        return int(round(self._d_t / self.base.d_t))

    def apply_base(self, cp, src, dst, t_start: float = 0.0) -> None:
        """dst = base(src) for a batch of device states (one application)."""
        n = self._base_steps()
        plan = self.base.plan(cp, src.shape[0])
        work = plan.new_state(2) if n > 1 else None
        plan.run(src, dst, n, t_start, self.base.d_t, save_every=n, work=work)

    def _plan_like(self, cp, batch: int):
        """Shape helper: (nx, ny, pitch) of this package's state layout."""
        from .codegen import lower_problem
        from .engine import state_pitch

        low = lower_problem(cp)
        if low.n_comp != 2 or low.x_dimension != 2:
            raise NotImplementedError("the CNN coarse operator handles 2-component 2D states")
        return low.nx, low.ny, state_pitch(low.ny)

    def coarse_propagator(self, cp, batch: int, n_steps: int):
        import torch

        nx, ny, pitch = self._plan_like(cp, batch)
        model = self.model
        model._ws(batch, nx, ny)  # allocate the activations up front
        tdt = torch.float32 if self.dtype == "f32" else torch.float64
        tmp = torch.empty((3, batch, 2, nx, pitch), dtype=tdt, device=model.device)
        op = self
        base_plan = None
        if self.base is not None:
            nb = self._base_steps()
            base_plan = self.base.plan(cp, batch)
            base_work = base_plan.new_state(2) if nb > 1 else None

        class _Prop:
            dtype = self.dtype

            def __call__(self_inner, src, dst, t_start):
                cur = src
                for k in range(n_steps):
                    out = dst if k == n_steps - 1 else tmp[k % 2]
                    res = None
                    if base_plan is not None:
                        res = tmp[2]
                        base_plan.run(cur, res, nb, t_start + k * op.d_t, op.base.d_t, save_every=nb, work=base_work)
                    model.forward(cur, out, nx, ny, residual=res)
                    cur = out

        return _Prop()

    def solve(self, ivp, parallel_enabled: bool = True) -> Solution:
        """Autoregressive application (supervised_ml_operator.py:91-128)."""
        import torch

        from .engine import StencilPlan, to_host
        from .codegen import lower_problem, FORWARD_EULER

        cp = ivp.constrained_problem
        t = discretize_time_domain(ivp.t_interval, self._d_t)
        nx, ny, pitch = self._plan_like(cp, 1)
        tdt = torch.float32 if self.dtype == "f32" else torch.float64
        states = torch.empty((len(t), 1, 2, nx, pitch), dtype=tdt, device=self.model.device)
        plan = StencilPlan(lower_problem(cp), FORWARD_EULER, self.dtype, 1)
        y0 = np.asarray(ivp.initial_condition.discrete_y_0(True), dtype=np.float64)
        plan.pack(y0[np.newaxis], states[0])
        prop = self.coarse_propagator(cp, 1, 1)
        for k in range(1, len(t)):
            prop(states[k - 1], states[k], float(t[k - 1]))
        y = plan.unpack(states[1:], len(t) - 1)
        return Solution(ivp, t[1:], to_host(y), vertex_oriented=True, d_t=self._d_t, copy=False)

    # ---- training on fine-solver trajectories
    def train(self, inputs, targets, nx: int, ny: int, epochs: int = 20, batch: int = 32, lr: float = 1e-3,
              seed: int = 0, lr_decay: float = 0.9, log=None, cp=None) -> List[float]:
        """Fits the model to (u(t), u(t + d_t)) pairs given as device states
        (N, 2, nx, pitch); returns the mean training loss of every epoch.
        With a base operator, ``cp`` is its constrained problem."""
        import torch

        if self.model is None:
            self.model = ResidualCNN(seed=seed, device=inputs.device)
        model = self.model
        n = inputs.shape[0]
        residual = inputs
        if self.base is not None:
            if cp is None:
                raise ValueError("training with a base operator needs the constrained problem")
            residual = torch.empty_like(inputs)
            chunk = 512
            for k0 in range(0, n, chunk):
                self.apply_base(cp, inputs[k0: k0 + chunk], residual[k0: k0 + chunk])
        u = inputs[:, :, :, :ny].double()
        du = (targets[:, :, :, :ny].double() - residual[:, :, :, :ny].double())
        s_in = 1.0 / torch.clamp(u.std(dim=(0, 2, 3)), min=1e-6)
        s_out = torch.clamp(du.std(dim=(0, 2, 3)), min=1e-12)
        model.set_scales(s_in.tolist(), s_out.tolist())
        gen = np.random.default_rng(seed)
        losses = []
        for ep in range(epochs):
            order = gen.permutation(n)
            tot = torch.zeros((), dtype=torch.float64, device=inputs.device)
            nb = 0
            rate = lr * (lr_decay ** ep)
            for k0 in range(0, n - batch + 1, batch):
                idx = torch.as_tensor(order[k0: k0 + batch], device=inputs.device)
                xb = inputs.index_select(0, idx)
                tb = targets.index_select(0, idx)
                rb = residual.index_select(0, idx) if self.base is not None else None
                yb = torch.empty_like(xb)
                model.forward(xb, yb, nx, ny, residual=rb)
                tot += model.loss_and_dy(yb, tb, nx, ny)
                model.backward(xb, nx, ny)
                model.adam_step(rate)
                nb += 1
            losses.append(float(tot.item()) / max(nb, 1))
            if log:
                log(f"epoch {ep}: loss {losses[-1]:.3e}")
        self.history = losses
        return losses


class CNNRegressor:
    """The residual CNN behind the regression-model contract of
    ``SupervisedMLOperator`` (scikit-learn's ``fit(x, y)`` / ``predict(x)``,
    supervised_ml_operator.py:238-284), for 2-component 2D problems at the
    vertices of ``cp``'s mesh.

    ``fit`` / ``predict`` take the reference's rows (one per vertex, the
    first 2 n_vertices columns the state at the step start in C order,
    identical for every row of a time point; the t / d_t / x columns are not
    used: the network is translation-invariant and time-invariant) or
    states of shape (N, *vertices, 2) (``layout="fields"`` data).  Training
    and prediction run on the GPU (``CNNCoarseOperator.train`` /
    ``coarse_propagator``); with ``base`` (a coarse ``FDMOperator`` whose step
    divides ``d_t``) the network learns a correction to it.
    """

    def __init__(self, cp, d_t: Optional[float] = None, *, base=None, epochs: int = 20, batch: int = 32,
                 lr: float = 1e-3, seed: int = 0, dtype: str = "float32", log=None):
        from .codegen import lower_problem

        low = lower_problem(cp)
        if low.n_comp != 2 or low.x_dimension != 2:
            raise NotImplementedError("the CNN regressor handles 2-component 2D problems")
        if base is not None and d_t is None:
            raise ValueError("a base operator needs the learned operator's d_t")
        self.cp = cp
        self.shape = tuple(low.vertices_shape)
        self.op = CNNCoarseOperator(d_t if d_t is not None else 1.0, base=base, dtype=dtype)
        self.epochs, self.batch, self.lr, self.seed, self.log = epochs, batch, lr, seed, log
        self.history: List[float] = []

    @property
    def n_vertices(self) -> int:
        return int(np.prod(self.shape))

    def _fields(self, x: np.ndarray) -> np.ndarray:
        if x.ndim == 2:
            n = self.n_vertices
            if x.shape[0] % n or x.shape[1] < 2 * n:
                raise ValueError(f"rows of {x.shape[1]} columns do not hold states of {n} vertices")
            return x[::n, :2 * n].reshape((-1,) + self.shape + (2,))
        if tuple(x.shape[1:]) != self.shape + (2,):
            raise ValueError(f"states of shape {tuple(x.shape[1:])} do not match {self.shape + (2,)}")
        return x

    def _states(self, fields: np.ndarray):
        import torch

        from .codegen import FORWARD_EULER, lower_problem
        from .engine import StencilPlan

        plan = StencilPlan(lower_problem(self.cp), FORWARD_EULER, self.op.dtype, len(fields))
        states = plan.new_state(1)[0]
        plan.pack_device(torch.from_numpy(np.ascontiguousarray(fields, dtype=np.float64)).to(plan.device), states)
        return plan, states

    def fit(self, x: np.ndarray, y: np.ndarray) -> "CNNRegressor":
        fields = self._fields(np.asarray(x))
        targets = np.asarray(y).reshape(fields.shape)
        _, inputs = self._states(fields)
        _, outs = self._states(targets)
        nx, ny = self.shape
        self.history = self.op.train(inputs, outs, nx, ny, epochs=self.epochs, batch=min(self.batch, len(fields)),
                                     lr=self.lr, seed=self.seed, log=self.log, cp=self.cp)
        return self

    def predict_fields(self, fields: np.ndarray) -> np.ndarray:
        """States (N, *vertices, 2) after one d_t."""
        import torch

        if self.op.model is None:
            raise ValueError("the regressor has not been fitted")
        plan, src = self._states(self._fields(np.asarray(fields)))
        dst = torch.empty_like(src)
        self.op.coarse_propagator(self.cp, src.shape[0], 1)(src, dst, 0.0)
        return plan.unpack(dst, src.shape[0]).cpu().numpy()

    def predict(self, x: np.ndarray) -> np.ndarray:
        x = np.asarray(x)
        out = self.predict_fields(self._fields(x))
        return out.reshape((-1, 2)) if x.ndim == 2 else out

    def rollout(self, y0: np.ndarray, n_steps: int) -> np.ndarray:
        """n_steps applications from y0 on the device: (n_steps, *vertices, 2)."""
        import torch

        if self.op.model is None:
            raise ValueError("the regressor has not been fitted")
        plan, s0 = self._states(np.asarray(y0)[np.newaxis])
        states = torch.empty((n_steps + 1,) + tuple(s0.shape), dtype=s0.dtype, device=s0.device)
        states[0].copy_(s0)
        prop = self.op.coarse_propagator(self.cp, 1, 1)
        for k in range(n_steps):
            prop(states[k], states[k + 1], k * self.op.d_t)
        return plan.unpack(states[1:], n_steps).cpu().numpy()

    def coarse_propagator(self, cp, batch: int, n_steps: int):
        """Batched device-to-device propagation (Parareal's coarse sweep)."""
        if self.op.model is None:
            raise ValueError("the regressor has not been fitted")
        return self.op.coarse_propagator(cp, batch, n_steps)
