"""Ensembles of initial value problems on meshes of different sizes.

The reference solves one IVP per ``FDMOperator.solve`` call
(``pararealml/operators/fdm/fdm_operator.py:48-77``); an ensemble there is a
Python loop.  Here the instances are grouped by constrained problem (same
equation, mesh and boundary conditions); every group is one batched
persistent-kernel plan, advanced with its own time step (e.g. set by a CFL
number on its mesh) for its own number of steps, and the step launches of
all groups are recorded into one CUDA graph, each group on its own stream so
that small meshes overlap large ones.  Replaying the graph advances the whole
ensemble; only the final states are kept.
"""

from __future__ import annotations

from typing import Dict, List, Sequence

import numpy as np

from .operators.fdm.fdm_operator import FDMOperator


class EnsembleSolver:
    def __init__(self, integrator, differentiator, *, dtype="float32", use_graph: bool = True):
        self._integrator = integrator
        self._differentiator = differentiator
        self._dtype = dtype
        self._use_graph = use_graph
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
            op = FDMOperator(self._integrator, self._differentiator, g["d_t"], dtype=self._dtype)
            plan = op.plan(g["cp"], len(g["members"]))
            y0 = np.stack([np.asarray(ivps[i].initial_condition.discrete_y_0(True), dtype=np.float64) for i in g["members"]])
            states = plan.new_state(1)
            plan.pack(y0, states[0])
            plan.autotune(g["d_t"], full=(n_steps == 1))
            g.update(op=op, plan=plan, n_steps=n_steps, y0=states[0], end=plan.new_state(1)[0],
                     work=plan.new_state(2) if n_steps > 1 else None, t0=float(t0),
                     stream=torch.cuda.Stream())
            self._groups.append(g)
        self._groups.sort(key=lambda g: -g["plan"].nx * g["plan"].ny)  # largest first
        self._graph = None

    def _issue(self) -> None:
        import torch

        main = torch.cuda.current_stream()
        for g in self._groups:
            g["stream"].wait_stream(main)
            with torch.cuda.stream(g["stream"]):
                g["plan"].run(g["y0"], g["end"], g["n_steps"], g["t0"], g["d_t"], save_every=g["n_steps"], work=g["work"])
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
