"""Ensembles of initial value problems on meshes of different sizes.

The reference solves one IVP per ``FDMOperator.solve`` call
(``pararealml/operators/fdm/fdm_operator.py:48-77``); an ensemble there is a
Python loop.  Here the instances are grouped by constrained problem (same
equation, mesh and boundary conditions); every group is one batched plan,
advanced with its own time step (e.g. set by a CFL number on its mesh) for
its own number of steps.

``launch="persistent"``: ALL groups and ALL steps run in one cooperative
persistent kernel (``engine.MultiRun``): round r is step r of every group
with more than r steps, the round's tiles of every mesh size spread over
the whole grid from one work list, a grid barrier between rounds; its tile
is tuned over the whole ensemble.  ``launch="streams"``: one launch per step
and group, each group on its own stream.  ``launch="auto"`` (default) builds
both and keeps the one that advances this ensemble faster (timed once at
setup).  The chosen launches are recorded in a CUDA graph and replayed;
replaying the graph advances the whole ensemble; only the final states are
kept.
"""

from __future__ import annotations

from typing import Dict, List, Sequence

import numpy as np

from .operators.fdm.fdm_operator import FDMOperator


class EnsembleSolver:
    def __init__(self, integrator, differentiator, *, dtype="float32", use_graph: bool = True,
                 launch: str = "auto"):
        if launch not in ("persistent", "streams", "auto"):
            raise ValueError("launch must be 'persistent', 'streams' or 'auto'")
        self._integrator = integrator
        self._differentiator = differentiator
        self._dtype = dtype
        self._use_graph = use_graph
        self._launch = launch
        self._multi = None
        self._graph = None
        self._groups: List[dict] = []
        self.stats: Dict[str, float] = {}

    def setup(self, ivps: Sequence, d_ts: Sequence[float]) -> None:
        """Groups the IVPs (each with its own d_t) and allocates device states."""
        import torch

        by_cp: Dict[int, dict] = {}
        for idx, (ivp, d_t) in enumerate(zip(ivps, d_ts)):
            cp = ivp.constrained_problem
            g = by_cp.setdefault(id(cp), {"cp": cp, "d_t": float(d_t), "t_interval": tuple(ivp.t_interval), "members": []})
            if not np.isclose(g["d_t"], d_t) or tuple(ivp.t_interval) != g["t_interval"]:
                raise ValueError("IVPs sharing a constrained problem must share d_t and the time interval")
            g["members"].append(idx)
        self._groups = []
        self._n = len(ivps)
        for g in by_cp.values():
            t0, t1 = g["t_interval"]
            n_steps = int(round((t1 - t0) / g["d_t"]))
            if not np.isclose(n_steps * g["d_t"], t1 - t0):
                raise ValueError("each d_t must divide its time interval")
            op = FDMOperator(self._integrator, self._differentiator, g["d_t"], dtype=self._dtype,
                             multi_round=self._launch != "streams")
            plan = op.plan(g["cp"], len(g["members"]))
            y0 = np.stack([np.asarray(ivps[i].initial_condition.discrete_y_0(True), dtype=np.float64) for i in g["members"]])
            states = plan.new_state(1)
            plan.pack(y0, states[0])
            g.update(op=op, plan=plan, n_steps=n_steps, y0=states[0], t0=float(t0))
            self._groups.append(g)
        self._groups.sort(key=lambda g: -g["plan"].nx * g["plan"].ny)  # largest first
        from .engine import MultiRun
        from . import _native

        # one cooperative launch needs one generated module (one equation,
        # boundary kinds and precision) and at most MULTI_MAX_GROUPS groups
        persistent = (self._launch != "streams" and len(self._groups) <= _native.MULTI_MAX_GROUPS
                      and all(g["plan"].module is self._groups[0]["plan"].module for g in self._groups)
                      and not self._groups[0]["plan"].low.lap_idx and self._groups[0]["plan"].implicit is None)
        self._multi = None
        multi = None
        if persistent:
            for g in self._groups:
                g["main"] = g["plan"].new_state(2)  # the rounds ping-pong between two slots
                g["multi_end"] = g["main"][(g["n_steps"] - 1) & 1]
            try:
                multi = MultiRun([{"plan": g["plan"], "first": g["y0"], "main": g["main"],
                                   "n_steps": g["n_steps"], "t0": g["t0"], "dt": g["d_t"], "ping_pong": True}
                                  for g in self._groups])
            except NotImplementedError:  # no multi-round tile fits: one launch per step
                multi = None
        if multi is None or self._launch == "auto":
            for g in self._groups:
                plan = g["plan"]
                plan.autotune(g["d_t"], full=(g["n_steps"] == 1))
                g.update(streams_end=plan.new_state(1)[0], work=plan.new_state(2) if g["n_steps"] > 1 else None,
                         stream=torch.cuda.Stream())
        self._multi = multi
        if multi is not None and self._launch == "auto":
            # the autotuner's choice between the two launch forms
            t_multi = self._time_advance()
            self._multi = None
            t_streams = self._time_advance()
            self._multi = multi if t_multi <= t_streams else None
            self.stats.update(persistent_ms=t_multi * 1e3, streams_ms=t_streams * 1e3)
        for g in self._groups:
            g["end"] = g["multi_end"] if self._multi is not None else g["streams_end"]
        self._graph = None

    def _time_advance(self) -> float:
        """Seconds of one eager advance (after one untimed), CUDA events."""
        import torch

        self._issue()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        self._issue()
        b.record()
        b.synchronize()
        return a.elapsed_time(b) / 1e3

    @property
    def tile(self):
        """Tile of the persistent launch (None with one launch per step)."""
        return self._multi.tile if self._multi is not None else None

    def _issue(self) -> None:
        import torch

        if self._multi is not None:
            self._multi.launch()
            return
        main = torch.cuda.current_stream()
        for g in self._groups:
            g["stream"].wait_stream(main)
            with torch.cuda.stream(g["stream"]):
                g["plan"].run(g["y0"], g["streams_end"], g["n_steps"], g["t0"], g["d_t"], save_every=g["n_steps"],
                              work=g["work"])
        for g in self._groups:
            main.wait_stream(g["stream"])

    def advance(self) -> None:
        """Advances every instance from its initial state to its end time."""
        import torch

        if not self._use_graph:
            self._issue()
            return
        if self._graph is None:
            self._issue()  # eager first run: kernels loaded, nothing recorded
            graph = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                with torch.cuda.graph(graph, stream=side):
                    self._issue()
            torch.cuda.current_stream().wait_stream(side)
            self._graph = graph
            return
        self._graph.replay()

    def final_states(self) -> List[np.ndarray]:
        """Final states (float64, (*vertices, C)) in the order of the IVPs."""
        if self._multi is not None:
            self._multi.check_status()
        out: List[np.ndarray] = [None] * self._n
        for g in self._groups:
            y = g["plan"].unpack(g["end"], len(g["members"])).cpu().numpy()
            for k, i in enumerate(g["members"]):
                out[i] = y[k]
        return out

    def bytes_per_advance(self) -> int:
        """Algorithmic bytes of one advance: read + write of every state per step."""
        total = 0
        for g in self._groups:
            p = g["plan"]
            total += 2 * p.C * p.esize * p.nx * p.ny * len(g["members"]) * g["n_steps"]
        return total

    def vertex_updates_per_advance(self) -> int:
        return sum(g["plan"].nx * g["plan"].ny * len(g["members"]) * g["n_steps"] for g in self._groups)
