"""Host logic of the step loops that interleave device solves (CPU only).

`StencilPlan._run_jacobi` (LHS.Y_LAPLACIAN rows: one fused step launch, then
the Jacobi solve, per step) and `StencilPlan._run_implicit` (one secant
solve per step) decide which buffer every step reads and writes and which
half-step boundary table each call sees.  The device calls are replaced by
recorders here; the arithmetic is covered by the GPU tests.
"""

import ctypes

import pytest

from pararealml_gb300 import _native
from pararealml_gb300.engine import StencilPlan


class _Low:
    lap_idx = (1,)
    x_dimension = 2


class _Work(list):
    pass


class _Buf:
    def __init__(self, addr):
        self.addr = addr

    def data_ptr(self):
        return self.addr


def _plan(bc_stride):
    plan = object.__new__(StencilPlan)
    plan.low = _Low()
    plan.esize = 8
    plan.inst = 1000
    plan.batch = 2
    p = _native.StepParams()
    p.batch = 2
    p.bc_stride = bc_stride
    p.dirichlet = 1_000_000
    p.neumann = 2_000_000
    plan.params = p
    return plan


@pytest.mark.parametrize("bc_stride", [0, 96])
def test_jacobi_loop_buffers_and_tables(bc_stride):
    plan = _plan(bc_stride)
    calls = []

    def launch(tile, y0, y0_b, out, out_b, step_stride, wa, wb, n, every, t0, dt):
        calls.append(("step", y0, out, n, every, round(t0, 12), plan.params.dirichlet, plan.params.neumann))

    def jacobi(state, slot, batch):
        calls.append(("jacobi", state, slot, batch, plan.params.dirichlet))

    plan._launch = launch
    plan.anti_laplacian = jacobi
    work = _Work([_Buf(7000), _Buf(8000)])
    traj, es = 50_000, 8
    plan._run_jacobi((8, 8, 8), 100, 1000, traj, 1000, 2000, work, 6, 2, 0.5, 0.1)
    steps = [c for c in calls if c[0] == "step"]
    solves = [c for c in calls if c[0] == "jacobi"]
    assert len(steps) == len(solves) == 6
    # step s + 1 is saved when 2 divides it; the others alternate work buffers
    outs = [c[2] for c in steps]
    assert outs == [7000, traj, 7000, traj + 2000 * es, 7000, traj + 2 * 2000 * es]
    ins = [c[1] for c in steps]
    assert ins == [100] + outs[:-1]
    assert all(c[3] == 1 and c[4] == 1 for c in steps)
    assert [c[5] for c in steps] == [round(0.5 + k * 0.1, 12) for k in range(6)]
    # step s reads half-step tables 2s..2s+2; its Jacobi solve the table at t + dt
    bc = bc_stride * es
    assert [c[6] for c in steps] == [1_000_000 + 2 * k * bc for k in range(6)]
    assert [c[7] for c in steps] == [2_000_000 + 2 * k * bc for k in range(6)]
    assert [(c[1], c[2], c[3]) for c in solves] == [(o, 2, 2) for o in outs]
    assert [c[4] for c in solves] == [1_000_000 + 2 * k * bc for k in range(6)]
    # the tables are restored afterwards
    assert (plan.params.dirichlet, plan.params.neumann) == (1_000_000, 2_000_000)


def test_jacobi_loop_restores_tables_after_a_failure():
    plan = _plan(96)
    plan._launch = lambda *a: None

    def failing(state, slot, batch):
        raise _native.ConvergenceError("no convergence")

    plan.anti_laplacian = failing
    with pytest.raises(_native.ConvergenceError):
        plan._run_jacobi((8, 8, 8), 100, 1000, 50_000, 1000, 2000, _Work([_Buf(7), _Buf(8)]), 4, 1, 0.0, 0.1)
    assert (plan.params.dirichlet, plan.params.neumann) == (1_000_000, 2_000_000)


@pytest.mark.parametrize("bc_stride", [0, 64])
def test_implicit_loop_buffers_and_tables(bc_stride):
    plan = _plan(bc_stride)
    plan.low.lap_idx = ()
    calls = []

    def step(y, out, t, dt, slot_bytes, nb):
        calls.append((y, out, round(t, 12), dt, slot_bytes, nb, plan.params.dirichlet))

    plan._implicit_step = step
    work = _Work([_Buf(7000), _Buf(8000)])
    plan._run_implicit(100, 50_000, 2000, work, 4, 2, 1.0, 0.25)
    assert [c[1] for c in calls] == [7000, 50_000, 7000, 50_000 + 2000 * 8]
    assert [c[0] for c in calls] == [100, 7000, 50_000, 7000]
    assert [c[2] for c in calls] == [1.0, 1.25, 1.5, 1.75]
    assert all(c[4] == bc_stride * 8 and c[5] == 2 for c in calls)
    assert [c[6] for c in calls] == [1_000_000 + 2 * k * bc_stride * 8 for k in range(4)]
    assert plan.params.dirichlet == 1_000_000


def test_implicit_params_mirror_layout():
    """The ctypes mirror matches the C struct field by field (offsets of the
    header's natural layout)."""
    ip = _native.ImplicitParams
    assert ip.cstride.offset == 40 and ip.dirichlet.offset == 72 and ip.dx.offset == 104
    assert ctypes.sizeof(ip) == 112


def test_autotuner_screens_every_candidate_and_retimes_the_fastest(monkeypatch):
    """StencilPlan.autotune with the device calls replaced by a clock that
    charges each tile a fixed cost per step (and grid caps 1 % more): every
    (tile, grid cap) pair is screened with rounds of 16 steps, the three
    fastest are re-timed with longer rounds, the fastest tile wins with the
    full grid, the caller's grid cap is restored and the choice is cached."""
    import types

    import torch

    from pararealml_gb300 import engine

    clock = [0.0]

    class Event:
        def __init__(self, enable_timing=True):
            self.t = None

        def record(self, *a):
            self.t = clock[0]

        def synchronize(self):
            pass

        def elapsed_time(self, other):
            return other.t - self.t

    class Lib:
        def prml_kernel_occupancy(self, kernel, threads, occ):
            occ._obj.value = 4
            return 0

    class State:
        def zero_(self):
            return self

        def __getitem__(self, i):
            return _Buf(0)

    stored = {}
    monkeypatch.setattr(torch.cuda, "Event", Event)
    monkeypatch.setattr(torch.cuda, "get_device_properties", lambda dev: types.SimpleNamespace(multi_processor_count=152))
    monkeypatch.setattr(_native, "lib", lambda: Lib())
    monkeypatch.setattr(_native, "check", lambda rc, what: None)
    monkeypatch.setattr(engine, "_tune_cache_load", lambda: {})
    monkeypatch.setattr(engine, "_tune_cache_store", lambda key, entry: stored.update({key: entry}))

    tiles = [(16, 32, 128), (8, 64, 128), (4, 64, 128, 1, 0, "w"), (16, 32, 128, 2)]
    cost = dict(zip(tiles, (0.0060, 0.0059, 0.0061, 0.0070)))  # ms per step
    plan = object.__new__(StencilPlan)
    plan.tile = None
    plan._tuned, plan._tuned_ctas = {}, {}
    plan.module = types.SimpleNamespace(gen=types.SimpleNamespace(key="k", step_kernels={t: ("n", 0) for t in tiles}))
    plan.nz, plan.rows, plan.ny, plan.batch, plan.inst = 1, 1025, 1025, 1, 1
    plan.device = "cuda"
    plan.params = types.SimpleNamespace(bc_stride=7, max_ctas=5)
    plan.new_state = lambda n: State()
    plan._step_kernel = lambda tile: tile
    launches = []

    def launch(tile, y0, y0_b, out, out_b, step_stride, wa, wb, n, every, t0, dt):
        clock[0] += cost[tile] * n * (1.01 if plan.params.max_ctas else 1.0)
        launches.append((tile, n, plan.params.max_ctas))

    plan._launch = launch
    best = StencilPlan.autotune(plan, 1e-4, full=True)
    assert best == (8, 64, 128) and plan._tuned_ctas[True] == 0
    assert (plan.params.max_ctas, plan.params.bc_stride) == (5, 7)
    assert stored == {"k:1x1025x1025:b1:full:v3": {"tile": [8, 64, 128], "ctas": 0}}
    # screening: 4 tiles x 2 grid caps, one warm-up launch and three rounds of 16 each
    screened = {(t, c) for t, n, c in launches[:32]}
    assert len(screened) == 8 and all(n in (2, 16) for _, n, _ in launches[:32])
    # re-timing: only the three fastest pairs, in longer timings
    retimed = {(t, c) for t, n, c in launches[32:]}
    assert retimed == {((8, 64, 128), 0), ((8, 64, 128), 304), ((16, 32, 128), 0)}
    assert len(launches) - 32 == 3 * 3 * 16
