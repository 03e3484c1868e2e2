"""Benchmark of the fused FDM stencil path (one JSON line on rank 0).

Workload (default): 2D Cahn-Hilliard (d = 0.1, gamma = 0.01) on [0, 64]^2 at
1024 x 1024 cells (1025^2 vertices, 2 components), zero-flux Neumann faces,
c0 ~ U(-0.1, 0.1) i.i.d. from a fixed seed, mu0 from c0, RK4 with
dt = 1e-4 for 2000 steps, every step stored (the reference FDMOperator's
trajectory contract).  One bench step = one such solve.

* ``value``: algorithmic bytes 2 * C * sizeof(double) per vertex update
  divided by the device time of the float64 drop-in solve (the reference's
  arithmetic type), inputs resident in HBM, trajectory kept on the device.
* ``e2e``: the same metric through the public drop-in call
  ``FDMOperator(RK4(), ThreePointCentralDifferenceMethod(), 1e-4,
  dtype=float64).solve_into(ivp, out)``: float64 host initial state in,
  float64 host trajectory out (pinned host buffer), copies inside the timed
  region.
* ``roofline``: the float64 step kernel against HBM, plus its float64 pipe
  fraction against the multiply-add rate measured live on the same GPU
  (the float64 kernel is bound by that pipe on GB300).
* ``f32``: the float32 fused stencil on the same workload with its own
  roofline and its relative error against the float64 result.
* ``cpu_baseline``: the numpy restatement of the reference (``oracle/``)
  timed on a bounded sample of the same workload on one host core.

``--impl reference`` times that CPU implementation alone, as the reference
arm.  With ``torchrun`` and N GPUs each rank runs an independent replica
(a single solve does not shard) and ``value`` sums the ranks' throughput.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "Parareal time-to-1e-6 rel err (ML vs FDM coarse, 1 GB300); stencil HBM GB/s"
N_CELLS = 1024
LENGTH = 64.0
D_T = 1e-4
N_STEPS = 2000
SEED = 541016860
L2_BYTES = 129 * 1024 * 1024


def make_ivp(ns, n_cells=N_CELLS, t_end=N_STEPS * D_T):
    import problems

    return problems.cahn_hilliard_2d(ns, n=n_cells, length=LENGTH, t_end=t_end, seed=SEED)


def workload_config(extra=None):
    cfg = {
        "workload": "2D Cahn-Hilliard d=0.1 gamma=0.01, [0,64]^2 at 1024x1024 cells (1025^2 vertices, C=2), "
        "zero-flux Neumann, c0~U(-0.1,0.1) seed 541016860, RK4 dt=1e-4 x2000 steps, full trajectory",
        "vertices": (N_CELLS + 1) ** 2,
        "components": 2,
        "time_steps": N_STEPS,
        "l2": "flushed (256 MiB write) between timed solves; the float64 trajectory (33.6 GB) exceeds L2",
    }
    if extra:
        cfg.update(extra)
    return cfg


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._proc = None

    def start(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
        except OSError:
            self._proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def stop(self):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[3:7]) if v.lower() == "active"})
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons,
            "samples": len(self.rows),
        }


# ---------------------------------------------------------------- distributed
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------- CPU arm
def cpu_sample(n_time_steps: int):
    """Seconds for ``n_time_steps`` RK4 steps of the numpy restatement on this host."""
    import pararealml_gb300 as ns
    from oracle import fdm as orc

    ivp = make_ivp(ns)
    cp = ivp.constrained_problem
    y = ivp.initial_condition.discrete_y_0(True)
    stepper = orc.FDMStepper(cp, orc.RK4, D_T)
    stepper.step(0.0, y)  # warm
    t0 = time.perf_counter()
    for i in range(n_time_steps):
        y = stepper.step(i * D_T, y)
    dt = time.perf_counter() - t0
    return dt, n_time_steps


# float64 bytes per vertex update: read the 2-component state once, write it once
BYTES_PER_UPDATE = 2 * 2 * 8


def reference_arm(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    n_sample = args.ref_sample_steps
    for _ in range(args.warmup):
        cpu_sample(1)
    times = []
    for _ in range(args.steps):
        dt, n = cpu_sample(n_sample)
        times.append(dt / n)
    per_step = statistics.mean(times)
    v = (N_CELLS + 1) ** 2
    gbs = BYTES_PER_UPDATE * v / per_step / 1e9
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": gbs,
        "unit": "GB/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": per_step * N_STEPS * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": workload_config(),
        "sample": f"{n_sample} RK4 time steps per bench step, extrapolated linearly to {N_STEPS}",
        "cpu_baseline": {
            "value": gbs,
            "unit": "GB/s",
            "cores": 1,
            "kind": "port",
            "sample": f"{n_sample} of {N_STEPS} RK4 time steps of the 1025^2 state per bench step "
                      "(numpy restatement of the reference, float64, single-threaded)",
            "cell_updates_per_s": v / per_step,
        },
        "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm
# float64 instructions per vertex update of the fused-order Cahn-Hilliard
# step (interior vertex): two unscaled Laplacians (3 adds, 1 multiply-add
# each), the update c + (dt 0.1 / dx^2) lapr(mu) (1 multiply-add), and
# mu = (-0.01 / dx^2) lapr(c) + (c c) c - c (1 product, 2 multiply-adds);
# the constant coefficients are computed once per thread
F64_OPS_PER_UPDATE = 12


def _load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _traffic(kernel: str, steps_per_launch: int):
    """DRAM bytes (read + write) per launch of ``kernel`` from a committed
    ncu capture of that same kernel, or None when none matches."""
    try:
        with open(os.path.join(ROOT, "profiles", "stencil_traffic.json")) as f:
            prof = json.load(f)
    except (OSError, ValueError):
        return None
    entry = prof.get(kernel) if isinstance(prof, dict) else None
    if not entry or int(entry.get("steps_per_launch", 1)) != steps_per_launch:
        return None
    return int(entry["dram_bytes_read"]) + int(entry["dram_bytes_write"])


def gpu_arm(args):
    import ctypes

    import torch

    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import pararealml_gb300 as ns
    from pararealml_gb300 import _native, codegen
    from pararealml_gb300.operators import fdm

    _native.build()
    ivp = make_ivp(ns)
    cp = ivp.constrained_problem
    y0_host = np.ascontiguousarray(ivp.initial_condition.discrete_y_0(True))
    v = y0_host.shape[0] * y0_host.shape[1]
    C = 2

    def make_op(dtype, **kw):
        return fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), D_T, dtype=dtype, **kw)

    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    def device_solver(dtype, forced=None):
        op = make_op(dtype, tile=forced)
        plan = op.plan(cp, 1)
        state0 = plan.new_state(1)
        plan.pack(y0_host[np.newaxis], state0[0])
        traj = plan.new_state(args.time_steps)
        plan.autotune(D_T)
        # the step launches of one solve, recorded once as a CUDA graph
        graph = plan.capture(state0[0], traj, args.time_steps, 0.0, D_T, 1)
        return plan, graph.replay, traj

    def time_device(run, steps, warmup):
        for _ in range(warmup):
            run()
        torch.cuda.synchronize()
        total = 0.0
        for _ in range(steps):
            flush.fill_(1.0)
            barrier(world)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            run()
            b.record()
            b.synchronize()
            total += a.elapsed_time(b) / 1e3
        return total / steps

    forced = tuple(int(x) if x.lstrip("-").isdigit() else x for x in args.tile.split(",")) if args.tile else None
    dtype = args.dtype
    # headline: the float64 drop-in (the reference's arithmetic type)
    plan64, run64, traj64 = device_solver(dtype, forced)
    sampler = ClockSampler(local)
    sampler.start()
    sec64 = time_device(run64, args.steps, args.warmup)
    sampler.stop()
    sec64 = max_over_ranks(sec64, world)
    es = 8 if dtype == "f64" else 4
    alg_bytes = 2 * C * es * v * args.time_steps
    value = sum_over_ranks(alg_bytes / sec64 / 1e9, world)
    kernel64 = plan64.module.gen.step_kernels[plan64.last_tile][0]
    tb64 = codegen.tile_steps(plan64.last_tile)

    if args.device_only or args.time_steps != N_STEPS:
        if rank == 0:
            print(json.dumps({"device_only": True, "dtype": dtype, "ms_per_step": sec64 * 1e3, "value": value,
                              "unit": "GB/s", "tile": list(plan64.last_tile), "kernel": kernel64}), flush=True)
        return

    # FP64 issue rate of this GPU (the float64 kernel's compute roofline)
    rate = ctypes.c_double()
    _native.check(_native.lib().prml_measure_fp64_fma(ctypes.byref(rate), plan64.stream_handle()), "fp64 probe")
    fp64_peak = rate.value

    # the same solve in float32 (reported beside the float64 headline)
    plan32, run32, traj32 = device_solver("f32")
    sec32 = max_over_ranks(time_device(run32, args.steps, args.warmup), world)
    f32_final = plan32.unpack(traj32[-1], 1)
    f64_final = plan64.unpack(traj64[-1], 1)
    f32_err = float(torch.linalg.norm(f32_final - f64_final) / torch.linalg.norm(f64_final))
    kernel32 = plan32.module.gen.step_kernels[plan32.last_tile][0]
    tb32 = codegen.tile_steps(plan32.last_tile)
    del traj32, traj64, f32_final, f64_final
    torch.cuda.empty_cache()

    # the same solves as ONE cooperative multi-round launch (every step of
    # the trajectory in one kernel, a grid barrier between steps)
    multi = {}
    if not args.no_multi:
        from pararealml_gb300.engine import MultiRun

        for dt_name in ("f64", "f32"):
            try:
                mop = make_op(dt_name, multi_round=True)
                mplan = mop.plan(cp, 1)
                ms0 = mplan.new_state(1)
                mplan.pack(y0_host[np.newaxis], ms0[0])
                mtraj = mplan.new_state(N_STEPS)
                run = MultiRun([{"plan": mplan, "first": ms0[0], "main": mtraj, "n_steps": N_STEPS, "t0": 0.0,
                                 "dt": D_T, "ping_pong": False}])
                msec = max_over_ranks(time_device(run.launch, args.steps, args.warmup), world)
                run.check_status()
                es_ = 8 if dt_name == "f64" else 4
                multi[dt_name] = {"ms_per_step": msec * 1e3, "value": 2 * C * es_ * v * N_STEPS / msec / 1e9,
                                  "unit": "GB/s", "tile": list(run.tile), "launches_per_solve": 1}
                del mtraj, ms0, run
                torch.cuda.empty_cache()
            except Exception as e:  # a failure here must not cost the rest of the line
                multi[dt_name] = {"error": f"{type(e).__name__}: {e}"}

    peaks = _load_peaks()
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    def roofline(sec, es_, kernel, tb):
        launches = -(-N_STEPS // tb)
        per_launch = sec / launches
        bytes_per_launch = 2 * C * es_ * v * N_STEPS / launches
        achieved = bytes_per_launch / per_launch / 1e9
        return {
            "bound": "hbm",
            "achieved": achieved,
            "peak": hbm_peak,
            "unit": "GB/s",
            "frac": achieved / hbm_peak,
            "traffic": _traffic(kernel, tb),
            "peak_source": peak_src,
            "kernel": kernel,
            "bytes_per_launch": bytes_per_launch,
            "steps_per_launch": tb,
            "launch_us": per_launch * 1e6,
        }

    # e2e through the public drop-in call with host buffers (float64)
    op_e2e = make_op(dtype)
    try:
        # pinned host memory on huge pages: base-page pinned buffers of this
        # size alternate between full and about half the link's rate
        from pararealml_gb300.hostmem import PinnedHostBuffer

        host_buf = PinnedHostBuffer((N_STEPS,) + y0_host.shape, torch.float64)
        host_out, host_kind = host_buf.tensor, "huge-page pinned" if host_buf.huge_pages else "pinned"
    except (MemoryError, RuntimeError):
        host_buf = None
        host_out = torch.empty((N_STEPS,) + y0_host.shape, dtype=torch.float64, pin_memory=True)
        host_kind = "pinned"

    def e2e_run():
        # the drop-in call with a caller-owned pinned output: the initial
        # state goes host -> device, the trajectory streams device -> host
        # in chunks while the next chunk computes
        op_e2e.solve_into(ivp, host_out)
        torch.cuda.synchronize()

    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(max(1, args.warmup)):
        e2e_run()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_run()
    e2e_sec = max_over_ranks((time.perf_counter() - t0) / e2e_steps, world)
    e2e_value = sum_over_ranks(alg_bytes / e2e_sec / 1e9, world)
    h2d = int(y0_host.nbytes)
    d2h = int(host_out.numel() * 8)
    # the host link on this machine: a raw 1 GiB device-to-host copy into the
    # same buffer (the bound of the streamed trajectory)
    raw = torch.empty(1 << 27, dtype=torch.float64, device="cuda")
    dst = host_out.view(-1)[: raw.numel()]
    dst.copy_(raw, non_blocking=True)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(3):
        dst.copy_(raw, non_blocking=True)
    ev1.record()
    ev1.synchronize()
    raw_d2h_gbs = 3 * raw.numel() * 8 / (ev0.elapsed_time(ev1) / 1e3) / 1e9
    huge_fraction = host_buf.huge_page_fraction() if host_buf is not None else 0.0
    del raw, dst
    del host_out
    if host_buf is not None:
        host_buf.close()

    cpu = None
    if rank == 0 and not args.no_cpu:
        dt, n = cpu_sample(args.ref_sample_steps)
        cpu_gbs = BYTES_PER_UPDATE * v / (dt / n) / 1e9
        cpu = {
            "value": cpu_gbs,
            "unit": "GB/s",
            "cores": 1,
            "kind": "port",
            "sample": f"{n} of {N_STEPS} RK4 time steps of the 1025^2 state (numpy restatement of the reference, "
                      "float64, single-threaded)",
            "cell_updates_per_s": v / (dt / n),
        }

    if rank == 0:
        clocks = sampler.summary()
        roof = roofline(sec64, es, kernel64, tb64)
        f64_ops = F64_OPS_PER_UPDATE * v * N_STEPS / sec64
        if dtype == "f64":
            roof["fp64_pipe"] = {
                "instructions_per_vertex_update": F64_OPS_PER_UPDATE,
                "achieved_per_s": f64_ops,
                "peak_per_s": fp64_peak,
                "frac": f64_ops / fp64_peak,
                "peak_source": "measured live (prml_measure_fp64_fma)",
            }
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "GB/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": sec64 * 1e3,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": dtype,
            "data": "synthetic",
            "config": workload_config(),
            "parallelism": f"replicas x{world}",
            "tile": list(plan64.last_tile),
            "grid_cap": plan64.last_ctas,
            "cell_updates_per_s": value * 1e9 / (2 * C * es),
            "roofline": roof,
            "f32": {
                "ms_per_step": sec32 * 1e3,
                "value": 2 * C * 4 * v * N_STEPS / sec32 / 1e9,
                "unit": "GB/s",
                "tile": list(plan32.last_tile),
                "grid_cap": plan32.last_ctas,
                "rel_l2_vs_f64_final": f32_err,
                "roofline": roofline(sec32, 4, kernel32, tb32),
            },
            "multi_round": multi,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_sec * 1e3, "steps": e2e_steps,
                    "call": f"FDMOperator(RK4(), ThreePointCentralDifferenceMethod(), {D_T}, dtype={dtype!r})"
                            f".solve_into(ivp, {host_kind} float64 host buffer)",
                    "host_buffer": host_kind, "huge_page_fraction": huge_fraction,
                    "raw_d2h_gbs": raw_d2h_gbs, "d2h_gbs": d2h / e2e_sec / 1e9},
            "gpu_launches": (-(-N_STEPS // tb64)) * args.steps,
            "clocks": clocks,
        }
        if not args.no_parareal:
            line["parareal"] = parareal_section(args)
            line["ensemble"] = ensemble_section(args)
            line["anti_laplacian"] = anti_laplacian_section(args)
            line["implicit"] = implicit_section(args)
            line["batched_parareal"] = batched_parareal_section(args)
            line["diffusion_65"] = diffusion_65_section(args)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def parareal_section(args) -> dict:
    """Parareal time-to-1e-6 on 2D Cahn-Hilliard at 257^2 with the learned coarse operator.

    Problem: d = 0.1, gamma = 0.01 on [0, 64]^2 at 256 x 256 cells (257^2
    vertices), zero-flux Neumann, c0 ~ U(-0.1, 0.1) (seed 541016860), mu0
    from c0; t in [0, 3.2]; fine operator RK4 dt = 1e-3 (3200 steps) in
    compensated float32; 32 time slices.  Error = relative L2 of the final
    state against the float64 serial solve (the oracle-exact GPU path).
    Methods, each timed after warm-up (CUDA graphs recorded):
      serial_f64, serial_f32c: plain GPU FDM, one 3200-launch graph;
      parareal_fdm: coarse = forward Euler dt 0.02, compensated float32;
      parareal_fdm64: the same coarse step in float64;
      parareal_ml: coarse = residual CNN correction on forward Euler dt
        0.0125, trained on 4096 (u(t), u(t + 0.05)) pairs from 64 batched
        fine solves of other random initial states, with the float64 FDM
        coarse step as fallback when updates stop halving.
    Each Parareal method is measured two ways: (1) iteration by iteration
    with every slice's iterations allowed (the final border point is copied
    and an event recorded after each iteration's termination test), giving
    the error after every iteration and ``time_to_1e-6``, the wall time at
    the first iteration whose final-state error is at most 1e-6; (2) the
    self-terminating run at update-norm tolerance 1e-6 (time, iterations,
    error).
    """
    import torch

    import pararealml_gb300 as ns
    import problems
    from pararealml_gb300 import _native
    from pararealml_gb300.learned import CNNCoarseOperator, generate_pairs
    from pararealml_gb300.operators import fdm
    from pararealml_gb300.operators.parareal import PararealOperator

    _native.build()
    n, length, t_end, slices = 256, 64.0, 3.2, 32
    ivp = problems.cahn_hilliard_2d(ns, n=n, length=length, t_end=t_end, seed=SEED)
    cp = ivp.constrained_problem
    y0 = ivp.initial_condition.discrete_y_0(True)

    def fine(dtype):
        return fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 1e-3, dtype=dtype, trajectory="final")

    def fe(dt, dtype):
        return fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), dt, dtype=dtype)

    def timed(fn, reps=2):
        fn()
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        out = None
        for _ in range(reps):
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best, out

    out = {"workload": "2D Cahn-Hilliard 257^2, t in [0,3.2], fine RK4 dt 1e-3 (3200 steps), 32 slices, "
                       "error vs float64 serial solve", "target_rel_err": 1e-6}

    def serial(dtype):
        op = fine(dtype)
        plan = op.plan(cp, 1)
        s0 = plan.new_state(1)
        plan.pack(y0[np.newaxis], s0[0])
        end = plan.new_state(1)
        graph = plan.capture(s0[0], end, 3200, 0.0, 1e-3, 3200)
        sec, _ = timed(lambda: graph.replay())
        return sec, plan.unpack(end[0], 1).cpu().numpy()[0]

    sec64, ref = serial("f64")
    sec32c, y32c = serial("f32c")
    err = lambda y: float(np.linalg.norm(y - ref) / np.linalg.norm(ref))  # noqa: E731
    out["serial_f64"] = {"seconds": sec64, "rel_err": 0.0}
    out["serial_f32c"] = {"seconds": sec32c, "rel_err": err(y32c)}

    def parareal(coarse, fallback=None):
        res = {}
        # (1) iteration by iteration: all slices' iterations allowed
        op = PararealOperator(fine("float32c"), coarse, 1e-30, n_slices=slices, trajectory="final", fallback=fallback)
        op.run(cp, y0[np.newaxis], ivp.t_interval)  # eager warm-up
        op.run(cp, y0[np.newaxis], ivp.t_interval)  # records the graphs
        torch.cuda.synchronize()
        snaps, events = [], []
        plan = op._ws.fplan

        def monitor(i, u_end):
            snaps.append(u_end.clone())
            ev = torch.cuda.Event(enable_timing=True)
            ev.record()
            events.append(ev)

        start = torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        start.record()
        op.run(cp, y0[np.newaxis], ivp.t_interval, monitor=monitor)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        curve = [err(plan.unpack(u, 1, esize=8).cpu().numpy()[0]) for u in snaps]
        times = [start.elapsed_time(ev) / 1e3 for ev in events]
        hit = next((k for k, e in enumerate(curve) if e <= 1e-6), None)
        res["error_by_iteration"] = curve
        res["seconds_by_iteration"] = times
        res["all_iterations_seconds"] = wall
        res["time_to_1e-6"] = times[hit] if hit is not None else None
        res["iterations_to_1e-6"] = hit + 1 if hit is not None else None
        res["fallback_at_iteration"] = op.last_stats["fallback_at_iteration"]
        # (2) the self-terminating run at the configuration's tolerance
        op = PararealOperator(fine("float32c"), coarse, 1e-6, n_slices=slices, trajectory="final", fallback=fallback)
        sec, sol = timed(lambda: op.solve(ivp), reps=1)
        res["tol_1e-6_run"] = {"seconds": sec, "rel_err": err(sol.discrete_y()[-1]),
                               "iterations": op.last_stats["iterations"][0],
                               "fallback_at_iteration": op.last_stats["fallback_at_iteration"],
                               "update_norms": [float(np.max(h)) for h in op.last_stats["norm_history"]]}
        return res

    out["parareal_fdm"] = parareal(fe(0.02, "float32c"))
    # the same coarse step in float64: a coarse propagator without float32
    # rounding noise in its output (G(U^{k+1}) - G(U^k) is then a smooth
    # function of the border points)
    out["parareal_fdm64"] = parareal(fe(0.02, "float64"))
    y0s = np.stack([problems.cahn_hilliard_2d(ns, n=n, length=length, t_end=t_end, seed=1000 + k)
                    .initial_condition.discrete_y_0(True) for k in range(64)])
    t0 = time.perf_counter()
    x, tgt = generate_pairs(fine("float32"), cp, y0s, t_end, 0.05)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    ml = CNNCoarseOperator(0.05, base=fe(0.0125, "float32"))
    t0 = time.perf_counter()
    losses = ml.train(x, tgt, n + 1, n + 1, epochs=args.cnn_epochs, batch=32, lr=2e-3, lr_decay=0.85, cp=cp)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    del x, tgt
    out["parareal_ml"] = parareal(ml, fallback=fe(0.02, "float64"))
    out["parareal_ml"].update({"train_seconds": train_s, "datagen_seconds": gen_s, "pairs": 4096,
                               "epochs": args.cnn_epochs, "final_train_mse": losses[-1]})
    cands = {"serial_f32c": out["serial_f32c"]["seconds"] if out["serial_f32c"]["rel_err"] <= 1e-6 else None,
             "serial_f64": out["serial_f64"]["seconds"],
             "parareal_fdm": out["parareal_fdm"]["time_to_1e-6"],
             "parareal_fdm64": out["parareal_fdm64"]["time_to_1e-6"],
             "parareal_ml": out["parareal_ml"]["time_to_1e-6"]}
    out["fastest_to_1e-6"] = min((k for k, v in cands.items() if v is not None), key=lambda k: cands[k])
    return out


def anti_laplacian_section(args) -> dict:
    """LHS.Y_LAPLACIAN rows: the reference's Navier-Stokes example
    (examples/navier_stokes_fdm.py, 101 x 81 vertices, RK4, dt 0.05), its
    first 10 steps from rest; each step ends with a Jacobi solve of the
    stream function from numpy's random estimate to tol 1e-3 (thousands of
    iterations).  GPU: float64 (the reference's precision) and float32, under
    one seed; CPU: the oracle's numpy restatement, one step."""
    import time

    import numpy as np
    import torch

    import pararealml_gb300 as ns
    import problems
    from oracle import fdm as orc
    from pararealml_gb300.operators import fdm

    n_steps, d_t = 10, 0.05
    out = {"workload": "Navier-Stokes example, 101x81 vertices, RK4 dt 0.05, 10 steps from rest, Jacobi tol 1e-3"}
    v = 101 * 81
    for dtype in ("float64", "float32"):
        op = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), d_t, dtype=dtype)
        np.random.seed(problems.JACOBI_SEED)
        op.solve(problems.navier_stokes_example(ns, 2, d_t))  # compile, tune
        ivp = problems.navier_stokes_example(ns, n_steps, d_t)
        plan = op.plan(ivp.constrained_problem, 1)
        plan.jacobi_iterations.clear()
        np.random.seed(problems.JACOBI_SEED)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op.solve(ivp)
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        its = [i[0] for i in plan.jacobi_iterations]
        es = 8 if dtype == "float64" else 4
        per_it = sec / sum(its)
        out[dtype] = {
            "ms_per_step": sec / n_steps * 1e3,
            "jacobi_iterations_per_step": float(np.mean(its)),
            "us_per_jacobi_iteration": per_it * 1e6,
            # one Jacobi iteration reads the estimate and the right-hand side
            # and writes the new estimate: 3 words per vertex
            "algorithmic_gbs": 3 * es * v / per_it / 1e9,
        }
    if not args.no_cpu:
        ivp = problems.navier_stokes_example(ns, 1, d_t)
        np.random.seed(problems.JACOBI_SEED)
        st = orc.FDMStepper(ivp.constrained_problem, "rk4", d_t)
        y = np.array(ivp.initial_condition.discrete_y_0(True))
        t0 = time.perf_counter()
        st.step(0.0, y)
        sec = time.perf_counter() - t0
        out["cpu_baseline"] = {"kind": "port", "cores": 1, "sample": "1 step (numpy oracle, float64)",
                               "ms_per_step": sec * 1e3, "jacobi_iterations_per_step": st.jacobi_iterations[0],
                               "us_per_jacobi_iteration": sec / st.jacobi_iterations[0] * 1e6}
    return out


def diffusion_65_section(args) -> dict:
    """The reference's own CPU-runnable case: 2D diffusion on
    [0,10]^2 at 64 x 64 cells, zero Dirichlet, Gaussian peak 1 at (5, 5),
    forward Euler dt 0.0025, 800 steps, float64, every step returned.  GPU:
    the drop-in FDMOperator.solve (host Solution, launch-bound: 34 KB
    state); CPU: the oracle's numpy restatement, the whole solve."""
    import time

    import numpy as np
    import torch

    import pararealml_gb300 as ns
    import problems
    from oracle import fdm as orc
    from pararealml_gb300.operators import fdm

    out = {"workload": "diffusion 65^2, forward Euler dt 0.0025, 800 steps, float64, full trajectory"}
    try:
        ivp = problems.diffusion_2d(ns, n=64, t_end=2.0)
        op = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 0.0025)
        op.solve(ivp)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(3):
            t0 = time.perf_counter()
            y = op.solve(ivp).discrete_y()
            best = min(best, time.perf_counter() - t0)
        out["gpu_seconds"] = best
        if not args.no_cpu:
            t0 = time.perf_counter()
            want = orc.fdm_solve(ivp.constrained_problem, ivp.initial_condition.discrete_y_0(True), ivp.t_interval,
                                 0.0025, "fe")
            out["cpu_baseline"] = {"kind": "port", "cores": 1, "sample": "whole solve (numpy oracle)",
                                   "seconds": time.perf_counter() - t0}
            out["max_abs_diff_vs_oracle"] = float(np.abs(y - want).max())
    except Exception as e:  # a failure here must not cost the rest of the line
        out["error"] = f"{type(e).__name__}: {e}"
    return out


def batched_parareal_section(args) -> dict:
    """Batched Parareal on 2D diffusion, [0,10]^2 at 256 x 256
    cells, zero Dirichlet, 64 Gaussian initial conditions (means ~ U([2,8]^2),
    covariance s I with s ~ U(0.3, 1), peak 1; seed 890237211), t in [0, 4]
    in 32 slices, fine RK4 dt 1e-4 (1250 steps per slice), coarse forward
    Euler dt 2.5e-4 (the stated 1e-2 does not divide a slice and is
    unstable), tol 1e-6, float32 solvers with float64 corrections; against
    the serial float32 and float64 solves of all 64 (one batched plan each).
    Errors are reported in the section instead of ending the run."""
    import time

    import numpy as np
    import torch

    import pararealml_gb300 as ns
    import problems
    from pararealml_gb300.operators import fdm
    from pararealml_gb300.operators.parareal import PararealOperator

    n, slices, t_end, n_ic = 256, 32, 4.0, 64
    out = {"workload": "diffusion 257^2, 64 Gaussian ICs, t in [0,4], 32 slices, fine RK4 1e-4, coarse FE 2.5e-4, "
                       "tol 1e-6, float32 solvers, error vs float64 serial"}
    try:
        rng = np.random.default_rng(problems.SEEDS[1])
        means = rng.uniform(2.0, 8.0, (n_ic, 2))
        scales = rng.uniform(0.3, 1.0, n_ic)
        mesh = ns.Mesh([(0.0, 10.0), (0.0, 10.0)], [10.0 / n, 10.0 / n])
        bc = ns.DirichletBoundaryCondition(lambda x, t: np.zeros((len(x), 1)), is_static=True)
        cp = ns.ConstrainedProblem(ns.DiffusionEquation(2), mesh, [(bc, bc)] * 2)
        from pararealml_gb300.initial_condition import gaussian_initial_states

        # the 64 Gaussian initial states evaluated on the device
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        y0 = gaussian_initial_states(cp, [[(means[k], scales[k] * np.eye(2))] for k in range(n_ic)],
                                     [[2.0 * np.pi * scales[k]] for k in range(n_ic)])
        torch.cuda.synchronize()
        out["initial_states_seconds"] = time.perf_counter() - t0
        n_steps = int(round(t_end / 1e-4))

        def serial(dtype):
            op = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 1e-4, dtype=dtype,
                                 trajectory="final")
            plan = op.plan(cp, n_ic)
            s0 = plan.new_state(1)
            plan.pack_device(y0, s0[0])
            end = plan.new_state(1)
            plan.run(s0[0], end, 200, 0.0, 1e-4, 200)  # warm-up (compile, tune)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            plan.run(s0[0], end, n_steps, 0.0, 1e-4, n_steps)
            torch.cuda.synchronize()
            return time.perf_counter() - t0, plan.unpack(end[0], n_ic).cpu().numpy()

        sec64, ref = serial("float64")
        sec32, y32 = serial("float32")
        err = lambda y: float(np.linalg.norm(y - ref) / np.linalg.norm(ref))  # noqa: E731
        out["serial_f64"] = {"seconds": sec64}
        out["serial_f32"] = {"seconds": sec32, "rel_err": err(y32)}
        def parareal(dtype):
            fine = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 1e-4, dtype=dtype,
                                   trajectory="final")
            coarse = fdm.FDMOperator(fdm.ForwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 2.5e-4,
                                     dtype=dtype)
            op = PararealOperator(fine, coarse, 1e-6, n_slices=slices, trajectory="final")
            op.run(cp, y0, (0.0, t_end))  # warm-up (plans, graphs)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = op.run(cp, y0, (0.0, t_end))
            torch.cuda.synchronize()
            sec = time.perf_counter() - t0
            y = res["final"].cpu().numpy()
            its = list(np.asarray(op.last_stats["iterations"]).reshape(-1))
            return {"seconds": sec, "rel_err": err(y), "iterations_max": int(max(its)),
                    "iterations_mean": float(np.mean(its))}

        out["parareal_f32"] = parareal("float32")
        out["parareal_f64"] = parareal("float64")
        out["note"] = ("one GPU: the serial batched solve of all 64 initial states already fills the GPU, so "
                       "Parareal's extra iterations cost more than its slice parallelism saves; float32 "
                       "stencils end ~1e-4 from the float64 answer (second differences of smooth fields)")
    except Exception as e:  # a failure here must not cost the rest of the line
        out["error"] = f"{type(e).__name__}: {e}"
    return out


def implicit_section(args) -> dict:
    """Implicit integrators: backward Euler on the [0,10]^2 Gaussian diffusion problem
    at 257^2 vertices (dt = 1e-3, 0.65 dx^2, 10 steps; 14-36 secant
    iterations per step), each step the reference's
    element-wise secant solve (scipy.optimize.newton's method) over
    right-hand-side kernel evaluations, float64; CPU: the oracle's numpy
    restatement, one step.  Errors are reported in the section instead of
    ending the run."""
    import time

    import numpy as np
    import torch

    import pararealml_gb300 as ns
    import problems
    from oracle import fdm as orc
    from pararealml_gb300.operators import fdm

    n_steps, d_t = 10, 1e-3
    out = {"workload": "diffusion 257^2 on [0,10]^2 (Gaussian peak 1), backward Euler dt 1e-3, 10 steps, float64"}
    try:
        op = fdm.FDMOperator(fdm.BackwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), d_t)
        op.solve(problems.diffusion_2d(ns, n=256, t_end=2 * d_t))  # compile
        ivp = problems.diffusion_2d(ns, n=256, t_end=n_steps * d_t)
        plan = op.plan(ivp.constrained_problem, 1)
        plan.secant_iterations.clear()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op.solve(ivp)
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        its = [i[0] for i in plan.secant_iterations]
        out["gpu"] = {"ms_per_step": sec / n_steps * 1e3, "secant_iterations_per_step": float(np.mean(its)),
                      "us_per_secant_iteration": sec / sum(its) * 1e6}
        if not args.no_cpu:
            ivp1 = problems.diffusion_2d(ns, n=256, t_end=d_t)
            st = orc.FDMStepper(ivp1.constrained_problem, "be", d_t)
            y = np.array(ivp1.initial_condition.discrete_y_0(True))
            t0 = time.perf_counter()
            st.step(0.0, y)
            sec = time.perf_counter() - t0
            out["cpu_baseline"] = {"kind": "port", "cores": 1, "sample": "1 step (numpy oracle, float64)",
                                   "ms_per_step": sec * 1e3, "secant_iterations_per_step": st.secant_iterations[0],
                                   "us_per_secant_iteration": sec / st.secant_iterations[0] * 1e6}
    except Exception as e:  # a failure here must not cost the rest of the line
        out["error"] = f"{type(e).__name__}: {e}"
    return out


def ensemble_section(args) -> dict:
    """Uneven-size ensemble: 256 shallow-water instances on
    [0, 64]^2 meshes of 64, 128, 256 or 512 cells (seeded draw), zero-flux on
    h, Gaussian bumps, RK4 at CFL 0.4 per mesh to t = 1, float32; one advance
    = every instance from t = 0 to t = 1, replayed from one CUDA graph."""
    import torch

    import pararealml_gb300 as ns
    import problems
    from pararealml_gb300.ensemble import EnsembleSolver
    from pararealml_gb300.operators import fdm

    ivps, d_ts = problems.shallow_water_ensemble(ns)

    def timed(launch):
        solver = EnsembleSolver(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), dtype="float32", launch=launch)
        solver.setup(ivps, d_ts)
        for _ in range(3):
            solver.advance()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = max(2, args.steps)
        a.record()
        for _ in range(reps):
            solver.advance()
        b.record()
        b.synchronize()
        return solver, a.elapsed_time(b) / 1e3 / reps

    streams_solver, streams_sec = timed("streams")
    solver, persistent_sec = timed("persistent")
    # the solver's default (launch="auto") keeps the faster form
    if streams_sec < persistent_sec:
        solver, sec, form = streams_solver, streams_sec, "one launch per step and group (streams)"
    else:
        sec, form = persistent_sec, "one cooperative multi-round kernel"
    nbytes = solver.bytes_per_advance()
    peak = _peak_hbm()[0]
    sizes = {}
    for g in solver._groups:
        sizes[f"{g['plan'].nx}^2"] = {"instances": len(g["members"]), "steps": g["n_steps"], "d_t": g["d_t"]}
    return {
        "workload": "256 shallow-water instances, meshes {64,128,256,512}^2 cells on [0,64]^2, RK4 at CFL 0.4, t in [0,1]",
        "groups": sizes,
        "state_bytes": int(sum(g["plan"].inst * 4 * len(g["members"]) for g in solver._groups)),
        "ms_per_advance": sec * 1e3,
        "vertex_updates_per_s": solver.vertex_updates_per_advance() / sec,
        "algorithmic_gbs": nbytes / sec / 1e9,
        "hbm_frac": nbytes / sec / 1e9 / peak,
        "launches_per_advance": 1 if solver.tile is not None else sum(g["n_steps"] for g in solver._groups),
        "launch": form,
        "tile": list(solver.tile) if solver.tile is not None else None,
        "streams_ms_per_advance": streams_sec * 1e3,
        "persistent_ms_per_advance": persistent_sec * 1e3,
    }


def profile_cnn(args) -> None:
    """CNN training steps on a batch of 32 random 257^2 two-component states
    (the learned coarse operator's training shape), timed per phase."""
    import torch

    from pararealml_gb300 import _native
    from pararealml_gb300.learned import ResidualCNN

    _native.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    B, H, W, pitch = 32, 257, 257, 288
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn((B, 2, H, pitch), device="cuda", generator=g) * 0.3
    t = x + 0.01 * torch.randn((B, 2, H, pitch), device="cuda", generator=g)
    model = ResidualCNN(seed=0)
    y = torch.empty_like(x)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    times = []
    for it in range(args.steps + args.warmup):
        ev[0].record()
        model.forward(x, y, H, W)
        ev[1].record()
        model.loss_and_dy(y, t, H, W)
        model.backward(x, H, W)
        ev[2].record()
        model.adam_step(1e-3)
        ev[3].record()
        ev[3].synchronize()
        if it >= args.warmup:
            times.append([ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2]), ev[2].elapsed_time(ev[3])])
    fwd, bwd, opt = np.mean(times, axis=0)
    flops_fwd = 2 * 9 * (2 * 32 + 4 * 32 * 32 + 32 * 2) * B * H * W
    mid_fwd = 2 * 9 * 4 * 32 * 32 * B * H * W
    print(json.dumps({"batch": B, "grid": [H, W], "forward_ms": fwd, "backward_ms": bwd, "adam_ms": opt,
                      "forward_tflops": flops_fwd / fwd / 1e9, "mid_layers_forward_flops": mid_fwd,
                      "train_step_tflops": 3 * flops_fwd / (fwd + bwd) / 1e9}), flush=True)


def profile_jacobi(args) -> None:
    """Profiling mode for the anti-Laplacian: two steps of the reference's
    Navier-Stokes example in float64 (step kernels and Jacobi solves, for a
    launch list), then four capped solves (64 iterations each) of a 257^2
    float32 Poisson problem (the staged kernel, for a detailed capture)."""
    import numpy as np
    import torch

    import pararealml_gb300 as ns
    import problems
    from pararealml_gb300 import _native
    from pararealml_gb300.operators import fdm

    np.random.seed(problems.JACOBI_SEED)
    op = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.05)
    ivp_ns = problems.navier_stokes_example(ns, 2, 0.05)
    op.solve(ivp_ns)
    mesh = ([(0.0, 2.0), (0.0, 2.0)], [2.0 / 256, 2.0 / 256])
    ivp = problems.jacobi_system(ns, "CARTESIAN", 2, mesh=mesh)
    plan = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.01,
                           dtype="float32").plan(ivp.constrained_problem, 1)
    st = plan.new_state(1)
    st.zero_()
    init = np.random.default_rng(0).random((257, 257, 1))
    plan.jacobi_init = lambda shape: init
    plan.jacobi_tol, plan.jacobi_max_iterations = 0.0, 64
    for _ in range(4):
        try:
            plan.anti_laplacian(st[0])
        except _native.ConvergenceError:
            pass
    torch.cuda.synchronize()
    print(json.dumps({"profile_jacobi": "ok",
                      "navier_stokes_iterations": op.plan(ivp_ns.constrained_problem, 1).jacobi_iterations}), flush=True)


def profile_implicit(args) -> None:
    """Profiling mode for the implicit integrators: backward Euler on the
    [0,10]^2 Gaussian diffusion problem at 257^2 vertices, dt 1e-3 (the
    implicit section's workload), one 2-step solve to compile and tune, then
    one 4-step solve (for a launch list)."""
    import torch

    import pararealml_gb300 as ns
    import problems
    from pararealml_gb300.operators import fdm

    op = fdm.FDMOperator(fdm.BackwardEulerMethod(), fdm.ThreePointCentralDifferenceMethod(), 1e-3)
    op.solve(problems.diffusion_2d(ns, n=256, t_end=2e-3))
    ivp = problems.diffusion_2d(ns, n=256, t_end=4e-3)
    op.solve(ivp)
    torch.cuda.synchronize()
    print(json.dumps({"profile_implicit": "ok",
                      "secant_iterations": op.plan(ivp.constrained_problem, 1).secant_iterations}), flush=True)


def _peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-sample-steps", type=int, default=6)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-multi", action="store_true", help="skip the multi-round (one launch per solve) variant")
    ap.add_argument("--device-only", action="store_true", help="time the float32 device solve only (profiling)")
    ap.add_argument("--time-steps", type=int, default=N_STEPS, help="time steps per solve (profiling runs only)")
    ap.add_argument("--no-parareal", action="store_true", help="skip the Parareal time-to-1e-6 section")
    ap.add_argument("--parareal-only", action="store_true", help="run and print the Parareal section alone")
    ap.add_argument("--cnn-epochs", type=int, default=8)
    ap.add_argument("--profile-cnn", action="store_true", help="a few CNN training steps only (profiling)")
    ap.add_argument("--tile", default=None, help="force the headline step kernel's tile, e.g. 16,64,256 or 8,64,64,1,0,w (profiling)")
    ap.add_argument("--dtype", default="f64", choices=["f64", "f32"],
                    help="precision of the headline solve (f64: the reference's; f32 for profiling)")
    ap.add_argument("--profile-jacobi", action="store_true", help="a few anti-Laplacian solves only (profiling)")
    ap.add_argument("--profile-implicit", action="store_true", help="two short backward Euler solves only (profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    elif args.profile_cnn:
        profile_cnn(args)
    elif args.profile_jacobi:
        profile_jacobi(args)
    elif args.profile_implicit:
        profile_implicit(args)
    elif args.parareal_only:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"parareal": parareal_section(args), "ensemble": ensemble_section(args),
                          "anti_laplacian": anti_laplacian_section(args)}), flush=True)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
