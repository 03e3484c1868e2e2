"""Stencil plans: generated module + device tables + tuned launch shape.

A ``StencilPlan`` is built once per (constrained problem, integrator, dtype,
batch) and owns

* the run-time compiled module of fused step kernels for the equation
  (``codegen.generate_source`` -> NVRTC -> cubin cache),
* the device copies of the Dirichlet / Neumann face tables and vertex
  coordinates,
* the launch parameter block (``prml_step_params``), and
* the tile shape, chosen by timing every candidate on the actual problem
  (``autotune``) and remembered per problem size in a JSON cache.

All device work is issued through the C ABI of ``libprml_gb300.so`` on the
caller's current torch CUDA stream.
"""

from __future__ import annotations

import ctypes
import json
import os
import threading
from typing import Dict, Optional, Tuple

import numpy as np

from . import _native, codegen

_DTYPES = {"f32": 4, "f64": 8, "f32c": 4}
_module_lock = threading.Lock()
_modules: Dict[str, "_LoadedModule"] = {}
_tune_lock = threading.Lock()


def _addr(x) -> int:
    """Device address of a tensor, or the int address itself."""
    return x if isinstance(x, int) else int(x.data_ptr())


def torch_dtype(dtype: str):
    import torch

    return {"f32": torch.float32, "f64": torch.float64, "f32c": torch.float32}[dtype]


def normalize_dtype(dtype) -> str:
    import torch

    if dtype in ("f32", "float32", np.float32, torch.float32):
        return "f32"
    if dtype in ("f32c", "float32c", "float32-compensated"):
        return "f32c"
    if dtype in ("f64", "float64", np.float64, torch.float64, float, None):
        return "f64"
    raise ValueError(f"unsupported dtype {dtype!r}: use float32, float32-compensated or float64")


class _LoadedModule:
    def __init__(self, gen: codegen.GeneratedModule):
        lib = _native.lib()
        # float64 modules place every multiply-add explicitly (fused-order
        # modules) or have none (reference order): no automatic contraction,
        # so every kernel variant of a module rounds alike
        opts = "--fmad=false" if gen.dtype == "f64" else ""
        path = _native.jit_module(gen.source, gen.key, opts)
        handle = ctypes.c_void_p()
        _native.check(lib.prml_module_load(path.encode(), ctypes.byref(handle)), "module load")
        self.handle = handle
        self.gen = gen
        self.kernels: Dict[str, ctypes.c_void_p] = {}

    def kernel(self, name: str, smem: int) -> ctypes.c_void_p:
        k = self.kernels.get(name)
        if k is None:
            k = ctypes.c_void_p()
            _native.check(
                _native.lib().prml_module_kernel(self.handle, name.encode(), smem, ctypes.byref(k)),
                f"kernel {name}",
            )
            self.kernels[name] = k
        return k


def load_module(low: codegen.LoweredProblem, integrator: int, dtype: str, exact_div: bool = False,
                fast: bool = False, multi: bool = False) -> _LoadedModule:
    gen = codegen.generate_source(low, integrator, dtype, exact_div, fast, multi)
    with _module_lock:
        mod = _modules.get(gen.key)
        if mod is None:
            mod = _LoadedModule(gen)
            _modules[gen.key] = mod
        return mod


# trajectories up to this size come back to the host through page-locked
# memory (the link's rate instead of a pageable copy's)
PINNED_RESULT_BYTES = 1 << 30


def to_host(y) -> np.ndarray:
    """A fresh host numpy array (owned by the caller) with the contents of
    the device tensor ``y``: copied into page-locked memory from torch's
    caching host allocator when at most ``PINNED_RESULT_BYTES``, else
    through pageable memory."""
    import torch

    if y.numel() * y.element_size() <= PINNED_RESULT_BYTES:
        h = torch.empty(y.shape, dtype=y.dtype, pin_memory=True)
        h.copy_(y)
        return h.numpy()
    return y.cpu().numpy()


def state_pitch(ny: int, dtype: str = "f32") -> int:
    """Row pitch in elements: a multiple of 32 elements, so rows start on
    128-byte (float32) / 256-byte (float64) boundaries and states of either
    precision share one layout (element-wise precision casts stay flat)."""
    return _native.round_up(ny, 32)


def _tune_cache_path() -> str:
    return os.path.join(_native.JIT_CACHE_DIR, "autotune.json")


def _tune_cache_load() -> dict:
    try:
        with open(_tune_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _tune_cache_store(key: str, entry) -> None:
    with _tune_lock:
        data = _tune_cache_load()
        data[key] = entry
        os.makedirs(_native.JIT_CACHE_DIR, exist_ok=True)
        tmp = _tune_cache_path() + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(data, f)
        os.replace(tmp, _tune_cache_path())


def jacobi_coefficients(cs: str, d_x, axis_coords) -> np.ndarray:
    """Coefficient table of the Jacobi estimate (layout in the C header's
    ``prml_jacobi_params``), each entry the reciprocal of the quantity the
    reference divides by in ``_next_anti_laplacian_estimate``
    (numerical_differentiator.py:1115-1186), computed the same way."""
    all_d_x_sqr = np.square(np.asarray(d_x, dtype=np.float64))
    if cs == "CARTESIAN":
        return np.array([1.0 / (2.0 / all_d_x_sqr).sum()])
    r = np.asarray(axis_coords[0], dtype=np.float64)
    r_sqr = r**2
    if cs == "SPHERICAL":
        phi = np.asarray(axis_coords[2], dtype=np.float64)
        sin_phi = np.sin(phi)
        r_sqr_sin_phi_sqr = r_sqr[:, None] * sin_phi[None, :] ** 2
        denom = 2.0 / all_d_x_sqr[0] + 2.0 / (all_d_x_sqr[1] * r_sqr_sin_phi_sqr) + 2.0 / (
            all_d_x_sqr[2] * r_sqr[:, None])
        return np.concatenate([
            1.0 / (d_x[0] * r), 1.0 / r_sqr, np.cos(phi), 1.0 / (2.0 * d_x[2] * sin_phi),
            (1.0 / r_sqr_sin_phi_sqr).reshape(-1), (1.0 / denom).reshape(-1),
        ])
    step = 2.0 / all_d_x_sqr[0] + 2.0 / (all_d_x_sqr[1] * r_sqr)
    if cs == "CYLINDRICAL":
        step = step + 2.0 / all_d_x_sqr[2]
    return np.concatenate([1.0 / (2.0 * d_x[0] * r), 1.0 / r_sqr, 1.0 / step])


class StencilPlan:
    """Everything needed to launch fused FDM steps for one problem."""

    # secant iterations an implicit step issues between two reads of the
    # instances' finished counters
    IMPLICIT_BLOCK = 8

    def __init__(
        self,
        low: codegen.LoweredProblem,
        integrator: int,
        dtype: str,
        batch: int = 1,
        tile: Optional[Tuple[int, int, int]] = None,
        device=None,
        op_order: str = "fused",
        multi: bool = False,
    ):
        import torch

        if op_order not in ("fused", "reference"):
            raise ValueError("op_order must be 'fused' or 'reference'")
        self.op_order = op_order
        self.low = low
        self.integrator = integrator
        self.dtype = dtype
        self.esize = _DTYPES[dtype]
        self.batch = batch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        if integrator in codegen.IMPLICIT and dtype != "f64":
            raise NotImplementedError(
                "implicit integrators run in float64: the secant's absolute step tolerance "
                "(1.48e-8 by default) is below float32 resolution")
        # implicit integrators use only the module's right-hand-side kernel
        implicit = integrator in codegen.IMPLICIT
        self.module = load_module(low, codegen.FORWARD_EULER if implicit else integrator, dtype, exact_div=implicit,
                                  fast=(op_order == "fused"), multi=multi and not implicit)
        self.implicit = None  # secant settings (a, tol, max_iterations, crank_nicolson) of an implicit integrator
        self.secant_iterations = []  # per step of the latest run: iterations of each instance
        self.secant_warnings = []  # warnings of the latest run
        # storage rows: all rows of all planes (a 3D mesh's planes are stacked
        # rows, so packing and the state layout are those of a 2D mesh)
        self.nz, self.rows = low.nz, low.nx
        self.nx, self.ny, self.C = low.nx * low.nz, low.ny, low.n_comp
        # compensated float32 states carry a second plane per component with
        # the rounding remainder of every update (value = hi + lo)
        self.comp = dtype == "f32c"
        self.planes = 2 * self.C if self.comp else self.C
        self.pitch = state_pitch(self.ny, dtype)
        self.plane = self.nx * self.pitch
        self.inst = self.planes * self.plane  # elements per instance
        tdt = torch_dtype(dtype)
        dev = self.device
        self._dir = torch.tensor(np.array(low.dirichlet), dtype=tdt, device=dev)
        self._neu = torch.tensor(np.array(low.neumann), dtype=tdt, device=dev)
        self._c0 = torch.tensor(np.array(low.coord_k0), dtype=torch.float64, device=dev)
        self._c1 = torch.tensor(np.array(low.coord_k1), dtype=torch.float64, device=dev)
        self._c0f = self._c0.to(torch.float32)
        self._c1f = self._c1.to(torch.float32)
        cz = low.coord_kz if low.coord_kz is not None else np.zeros(1)
        self._cz = torch.tensor(np.array(cz), dtype=torch.float64, device=dev)
        self._czf = self._cz.to(torch.float32)
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.params = self._base_params()
        self.params.status = self._status.data_ptr()
        # LHS.Y_LAPLACIAN components: a Jacobi solve after every step
        self.jacobi_tol = 1e-3
        self.jacobi_max_iterations = 1_000_000
        # source of each solve's initial estimate: the reference draws it from
        # numpy's global generator (numerical_differentiator.py:910-911)
        self.jacobi_init = np.random.random
        self.jacobi_iterations = []  # per solve of the latest run: iterations of each instance
        if low.lap_idx:
            self._jacobi_setup()
        if integrator in codegen.IMPLICIT:
            self._implicit_setup()
        self.tile = tuple(tile) if tile is not None else None  # forced by the caller
        self._tuned: Dict[bool, Tuple[int, ...]] = {}  # trajectory pattern -> tuned tile
        self._tuned_ctas: Dict[bool, int] = {}  # trajectory pattern -> tuned grid cap (0 = fill the GPU)
        self._user_ctas = 0
        self.last_tile: Optional[Tuple[int, ...]] = self.tile
        self.last_ctas = 0  # grid cap of the latest run (0 = every resident CTA)
        if self.tile is not None and self.tile not in self.module.gen.step_kernels:
            raise ValueError(f"tile {self.tile} is not instantiated for this module")

    # ------------------------------------------------------------------
    def _base_params(self) -> _native.StepParams:
        low = self.low
        p = _native.StepParams()
        p.cstride = self.plane
        p.pitch = self.pitch
        p.nx, p.ny = self.rows, self.ny
        p.nz, p.tile_z, p.box_planes = self.nz, 1, 1
        p.batch = self.batch
        p.face_len = low.face_len
        p.elem_bytes = self.esize
        p.dirichlet = self._dir.data_ptr()
        p.neumann = self._neu.data_ptr()
        p.coord0 = self._c0.data_ptr()
        p.coord1 = self._c1.data_ptr()
        d0, d1 = low.dx_k
        p.inv_2dx0, p.inv_2dx1 = 1.0 / (2.0 * d0), 1.0 / (2.0 * d1)
        p.inv_dxx0, p.inv_dxx1 = 1.0 / (d0 * d0), 1.0 / (d1 * d1)
        p.two_dx0, p.two_dx1 = 2.0 * d0, 2.0 * d1
        p.coord0_f = self._c0f.data_ptr()
        p.coord1_f = self._c1f.data_ptr()
        # ctypes rounds each double to the nearest float, like a device cast
        p.inv_2dx0_f, p.inv_2dx1_f = p.inv_2dx0, p.inv_2dx1
        p.inv_dxx0_f, p.inv_dxx1_f = p.inv_dxx0, p.inv_dxx1
        p.two_dx0_f, p.two_dx1_f = p.two_dx0, p.two_dx1
        dz = low.dx_z
        p.inv_2dx2, p.inv_dxx2, p.two_dx2 = 1.0 / (2.0 * dz), 1.0 / (dz * dz), 2.0 * dz
        p.dxx0, p.dxx1, p.dxx2 = d0 * d0, d1 * d1, dz * dz
        p.inv_2dx2_f, p.inv_dxx2_f, p.two_dx2_f = p.inv_2dx2, p.inv_dxx2, p.two_dx2
        p.coord2 = self._cz.data_ptr()
        p.coord2_f = self._czf.data_ptr()
        return p

    def new_state(self, n: int = 1):
        """Uninitialised device states, shape (n, batch, C, nx, pitch)."""
        import torch

        return torch.empty(
            (n, self.batch, self.planes, self.nx, self.pitch), dtype=torch_dtype(self.dtype), device=self.device
        )

    def limit_ctas(self, max_ctas: int) -> None:
        """Caps the persistent grid (0 = as many CTAs as fit on the GPU, or
        the cap the autotuner found best for the problem)."""
        self._user_ctas = int(max_ctas)
        self.params.max_ctas = int(max_ctas)

    def set_t_offset(self, t_offset) -> None:
        """Per-instance time offsets (device float64 tensor of length batch) or None."""
        self._t_offset = t_offset
        self.params.t_offset = 0 if t_offset is None else t_offset.data_ptr()

    @staticmethod
    def stream_handle() -> int:
        import torch

        return torch.cuda.current_stream().cuda_stream

    # ------------------------------------------------------------------
    def pack(self, y_host: np.ndarray, out) -> None:
        """Host float64 (batch, *vertices, C) -> device state ``out`` (batch, C, nx, pitch)."""
        import torch

        y = torch.from_numpy(np.ascontiguousarray(y_host, dtype=np.float64)).to(self.device, non_blocking=False)
        self.pack_device(y, out)

    def pack_device(self, y, out, esize: Optional[int] = None) -> None:
        """Device float64 (batch', *vertices, C) -> device state (batch', C, nx, pitch)
        in this plan's precision, or to a plain state of ``esize`` bytes per element."""
        batch = y.shape[0]
        nv = self.nx * self.ny
        es, comp, inst = (self.esize, int(self.comp), self.inst) if esize is None else (esize, 0, self.C * self.plane)
        _native.check(
            _native.lib().prml_pack(
                y.data_ptr(), out.data_ptr(), es, batch, self.C, self.nx, self.ny,
                self.pitch, nv * self.C, inst, comp, self.stream_handle(),
            ),
            "pack",
        )

    def unpack(self, state, n_inst: int, esize: Optional[int] = None):
        """Device states (n_inst instances) -> device float64 (n_inst, *vertices, C)."""
        import torch

        out = torch.empty((n_inst,) + tuple(self.low.vertices_shape) + (self.C,), dtype=torch.float64, device=self.device)
        self.unpack_into(state, n_inst, out, esize)
        return out

    def unpack_into(self, state, n_inst: int, out, esize: Optional[int] = None) -> None:
        """Like ``unpack``, into the device float64 buffer ``out`` (at least n_inst states)."""
        es, comp, inst = (self.esize, int(self.comp), self.inst) if esize is None else (esize, 0, self.C * self.plane)
        nv = self.nx * self.ny
        done = 0
        while done < n_inst:
            n = min(65535, n_inst - done)
            _native.check(
                _native.lib().prml_unpack(
                    state.data_ptr() + done * inst * es, es,
                    out.data_ptr() + done * nv * self.C * 8, n, self.C, self.nx, self.ny,
                    self.pitch, inst, nv * self.C, comp, self.stream_handle(),
                ),
                "unpack",
            )
            done += n

    def run_to_host(self, y0, host_out, n_steps: int, t0: float, dt: float, save_every: int = 1,
                    chunk_saves: Optional[int] = None) -> None:
        """``n_steps`` fused steps from device state ``y0``, every saved step
        streamed to ``host_out`` (pinned float64, (n_saved, batch, *vertices, C)).

        The trajectory is computed in chunks of ``chunk_saves`` saved steps
        (about 1 GiB of float64 by default) into two device buffers; each
        chunk is converted to float64 and copied to the host on a copy
        stream while the next chunk computes, so the device holds four
        chunk buffers however long the trajectory is (kept by the plan for
        its next streamed run).  Returns when the last copy has landed.
        """
        import torch

        if n_steps % save_every != 0:
            raise ValueError("n_steps must be a multiple of save_every")
        n_save = n_steps // save_every
        per_save = self.batch * self.nx * self.ny * self.C * 8
        if tuple(host_out.shape) != (n_save, self.batch) + tuple(self.low.vertices_shape) + (self.C,):
            raise ValueError(f"host_out must have shape {(n_save, self.batch) + tuple(self.low.vertices_shape) + (self.C,)}")
        if host_out.dtype != torch.float64 or host_out.device.type != "cpu":
            raise ValueError("host_out must be a float64 host tensor (pinned for overlap)")
        if n_save == 0:
            return
        chunk = max(1, min(n_save, chunk_saves or (1 << 30) // per_save))
        # the chunk buffers (about 4 GiB) are kept for the plan's next call:
        # repeated streamed solves allocate nothing
        cached = getattr(self, "_host_chunks", None)
        if cached is None or cached[0] != chunk:
            self._host_chunks = None
            cached = (chunk, [self.new_state(chunk), self.new_state(chunk)],
                      [torch.empty((chunk * self.batch,) + tuple(self.low.vertices_shape) + (self.C,),
                                   dtype=torch.float64, device=self.device) for _ in range(2)])
            self._host_chunks = cached
        _, dev, stage = cached
        work = self.new_state(2) if save_every > 1 else None
        main = torch.cuda.current_stream()
        copier = torch.cuda.Stream()
        copied = [None, None]
        cur = y0
        for ci, s in enumerate(range(0, n_save, chunk)):
            k = ci & 1
            m = min(chunk, n_save - s)
            self.run(cur, dev[k], m * save_every, t0 + s * save_every * dt, dt, save_every, work=work)
            if copied[k] is not None:
                main.wait_event(copied[k])  # staging buffer k is free again
            self.unpack_into(dev[k], m * self.batch, stage[k])
            ready = torch.cuda.Event()
            ready.record(main)
            copier.wait_event(ready)
            with torch.cuda.stream(copier):
                host_out[s : s + m].view(-1).copy_(stage[k][: m * self.batch].view(-1), non_blocking=True)
                done = torch.cuda.Event()
                done.record(copier)
            copied[k] = done
            cur = dev[k][m - 1]
        for ev in copied:
            if ev is not None:
                ev.synchronize()

    # ------------------------------------------------------------------
    def _jacobi_setup(self) -> None:
        """Parameters, coefficient tables and scratch of the anti-Laplacian
        solve (``prml_anti_laplacian``)."""
        import torch

        low = self.low
        if low.x_dimension == 0:
            raise NotImplementedError("LHS.Y_LAPLACIAN needs a spatial mesh")
        if len(low.lap_idx) > 16:
            raise NotImplementedError("at most 16 LHS.Y_LAPLACIAN components are supported")
        if self.batch > _native.JACOBI_MAX_BATCH:
            raise NotImplementedError(
                f"LHS.Y_LAPLACIAN problems run at most {_native.JACOBI_MAX_BATCH} instances per plan")
        cp_mesh_dx = list(low.mesh_dx)
        d = low.x_dimension
        first = 3 - d
        n = [1, 1, 1]
        n[first:] = list(low.vertices_shape)
        jp = _native.JacobiParams()
        for a in range(3):
            jp.n[a] = n[a]
        jp.first_axis = first
        jp.coord_system = {"CARTESIAN": 0, "POLAR": 1, "CYLINDRICAL": 2, "SPHERICAL": 3}[low.cs]
        jp.comps = self.C
        jp.n_lap = len(low.lap_idx)
        for k, c in enumerate(low.lap_idx):
            jp.lap_comp[k] = c
        jp.elem_bytes = self.esize
        jp.batch = self.batch
        jp.pitch = self.pitch
        jp.face_len = low.face_len
        jp.face_base = 0 if d == 3 else 2
        jp.cstride = self.plane
        jp.inst = self.inst
        jp.dir_mask = low.dir_mask
        jp.neu_mask = low.neu_mask
        for a in range(3):
            h = cp_mesh_dx[a - first] if a >= first else 1.0
            jp.inv_dxx[a] = 1.0 / (h * h)
            jp.two_dx[a] = 2.0 * h
        coef = jacobi_coefficients(low.cs, cp_mesh_dx, low.axis_coords)
        self._jcoef = torch.tensor(coef, dtype=torch_dtype(self.dtype), device=self.device)
        jp.coef = self._jcoef.data_ptr()
        jp.dirichlet = self._dir.data_ptr()
        jp.neumann = self._neu.data_ptr()
        jp.tol = float(self.jacobi_tol)
        jp.max_iterations = int(self.jacobi_max_iterations)
        self._jp = jp
        nbytes = int(_native.load_library().prml_jacobi_scratch_bytes(ctypes.byref(jp)))
        if nbytes < 0:
            _native.check(_native.PRML_ERR_ARG, "anti-Laplacian parameters")
        self._jscratch = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        v = int(np.prod(low.vertices_shape))
        self._jinit_host = torch.empty((self.batch, v * jp.n_lap), dtype=torch.float64).pin_memory()
        self._jinit = torch.empty((self.batch, v * jp.n_lap), dtype=torch.float64, device=self.device)

    def anti_laplacian(self, state, table_slot: int = 0, batch: Optional[int] = None) -> None:
        """Replaces the LHS.Y_LAPLACIAN planes of the device state ``state``
        (their right-hand side on entry) by the Jacobi solution, constrained
        by boundary table ``table_slot`` (time-dependent conditions: half step
        k of the current run).  Each instance's initial estimate is drawn
        from ``jacobi_init`` with the reference's shape (*vertices, n_lap)."""
        jp = self._jp
        nb = self.batch if batch is None else batch
        shape = tuple(self.low.vertices_shape) + (jp.n_lap,)
        for b in range(nb):
            self._jinit_host[b].numpy()[:] = np.asarray(self.jacobi_init(shape), dtype=np.float64).reshape(-1)
        self._jinit[:nb].copy_(self._jinit_host[:nb], non_blocking=True)
        jp.batch = nb
        jp.tol = float(self.jacobi_tol)
        jp.max_iterations = int(self.jacobi_max_iterations)
        off = int(table_slot) * int(self.params.bc_stride) * self.esize
        jp.dirichlet = self.params.dirichlet + off
        jp.neumann = self.params.neumann + off
        its = (ctypes.c_longlong * nb)()
        try:
            _native.check(
                _native.lib().prml_anti_laplacian(
                    ctypes.byref(jp), _addr(state), self._jinit.data_ptr(), self._jscratch.data_ptr(),
                    self._jscratch.numel(), its, self.stream_handle(),
                ),
                "anti-Laplacian",
            )
        finally:
            jp.batch = self.batch
            self.jacobi_iterations.append(list(its))
            if len(self.jacobi_iterations) > 65536:  # direct calls outside run(): keep the latest
                del self.jacobi_iterations[:-32768]

    def _run_jacobi(self, tile, y0, y0_bstride, traj, traj_bstride, traj_step_stride, work, n_steps,
                    save_every, t0, dt) -> None:
        """Steps of a problem with LHS.Y_LAPLACIAN components: one fused step
        launch, then the Jacobi solve on its output, per step."""
        es = self.esize
        base_dir, base_neu = self.params.dirichlet, self.params.neumann
        bc_bytes = int(self.params.bc_stride) * es
        cur, cur_bstride = y0, y0_bstride
        try:
            for s in range(n_steps):
                step = s + 1
                if step % save_every == 0:
                    out = traj + (step // save_every - 1) * traj_step_stride * es
                    out_bstride = traj_bstride
                else:
                    out, out_bstride = _addr(work[s & 1]), self.inst
                # step s reads the tables of half steps 2s .. 2s + 2
                self.params.dirichlet = base_dir + 2 * s * bc_bytes
                self.params.neumann = base_neu + 2 * s * bc_bytes
                self._launch(tile, cur, cur_bstride, out, out_bstride, self.params.batch * out_bstride,
                             0, 0, 1, 1, t0 + s * dt, dt)
                if out_bstride != self.inst:
                    raise NotImplementedError("the anti-Laplacian solve needs the plan's instance stride")
                self.anti_laplacian(out, 2, self.params.batch)
                cur, cur_bstride = out, out_bstride
        finally:
            self.params.dirichlet, self.params.neumann = base_dir, base_neu

    def _implicit_setup(self) -> None:
        import torch

        low = self.low
        ip = _native.ImplicitParams()
        d = low.x_dimension
        n = [1, 1, 1]
        if d:
            n[3 - d:] = list(low.vertices_shape)
        for a in range(3):
            ip.n[a] = n[a]
        ip.first_axis = 3 - d
        ip.comps = self.C
        ip.batch = self.batch
        ip.pitch = self.pitch
        ip.face_len = low.face_len
        ip.face_base = 0 if d == 3 else 2
        ip.cstride = self.plane
        ip.inst = self.inst
        ip.d_mask = sum(1 << c for c in low.d_idx)
        ip.dir_mask = low.dir_mask
        ip.dx = float(np.finfo(float).eps ** 0.33)
        self._ip = ip
        # the reference's defaults (numerical_integrator.py:140, 232); the
        # operator replaces them with its integrator's settings
        self.implicit = {"a": 0.5 if self.integrator == codegen.CRANK_NICOLSON else 1.0, "tol": 1.48e-8,
                         "max_iterations": 50, "crank_nicolson": self.integrator == codegen.CRANK_NICOLSON}
        self._isec = self.new_state(8)  # p, p1, q0, q1, fu, f, result, f at the step start
        self._iflags = torch.empty(self.batch * self.inst, dtype=torch.uint8, device=self.device)
        self._icount = torch.zeros((self.batch, 4), dtype=torch.int32, device=self.device)
        self._istat = torch.zeros((self.batch, 4), dtype=torch.float64, device=self.device)
        self._iits = torch.zeros(self.batch, dtype=torch.int32, device=self.device)
        self._iiter = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._implicit_stream = torch.cuda.Stream(device=self.device)

    def _implicit_step(self, y: int, out: int, t: float, dt: float, slot_bytes: int, nb: int) -> None:
        """One backward Euler / Crank-Nicolson step from the device state at
        address ``y`` to ``out`` (numerical_integrator.py:199-270): forward
        Euler predictor, then the element-wise secant iteration of
        scipy.optimize.newton on the residual, every instance stopping on its
        own.  The stop test, the result copy, the status sums and the
        iteration count run on the device (``prml_implicit_stop``), and the
        buffer roles repeat every two iterations, so two iterations are
        recorded once per step as a CUDA graph and replayed; the host reads
        the instances' finished counters every ``IMPLICIT_BLOCK`` iterations
        (iterations of finished instances leave them unchanged) and raises
        the reference's warnings and error from each instance's recorded
        status, in the order the instances stopped.  ``self.params`` tables
        point at the step start (half step 0)."""
        import warnings

        import torch

        lib = _native.lib()
        ip = self._ip
        s = self.implicit
        ip.batch = nb
        ip.dt = float(dt)
        ip.a = s["a"]
        ip.tol = s["tol"]
        ip.crank_nicolson = int(s["crank_nicolson"])
        base_dir, base_neu = self.params.dirichlet, self.params.neumann
        ip.dirichlet = base_dir + 2 * slot_bytes  # constraints at t + dt
        bufs = [self._isec[k].data_ptr() for k in range(4)]  # p, p1, q0, q1 (roles swap)
        fu, f, f0 = self._isec[4].data_ptr(), self._isec[5].data_ptr(), self._isec[7].data_ptr()
        res = self._isec[6].data_ptr()
        cnt, stats, its_dev, counter = self._icount, self._istat, self._iits, self._iiter
        flags = self._iflags.data_ptr()
        batch_saved = self.params.batch
        self.params.batch = nb

        def rhs_at(state, dst, when, slot):
            self.params.dirichlet = base_dir + slot * slot_bytes
            self.params.neumann = base_neu + slot * slot_bytes
            self.rhs(state, dst, when)

        def residual(xi, qi, prev):
            rhs_at(bufs[xi], f, t + dt, 2)
            _native.check(lib.prml_implicit_residual(
                ctypes.byref(ip), bufs[xi], y, f, fu, bufs[qi], 0 if prev is None else bufs[prev],
                cnt.data_ptr(), self.stream_handle()), "implicit residual")

        def stop(xs, xo, force):
            _native.check(lib.prml_implicit_stop(
                ctypes.byref(ip), bufs[xs], bufs[xo], flags, cnt.data_ptr(), counter.data_ptr(), force, res,
                stats.data_ptr(), its_dev.data_ptr(), self.stream_handle()), "implicit stop")

        def iteration(roles, last):
            """One secant iteration from the buffer roles (p, p1, q0, q1);
            ``last``: the iteration limit, the instances still running stop
            on the previous iterate.  Returns the next roles."""
            p_, p1_, q0_, q1_ = roles
            _native.check(lib.prml_implicit_update(
                ctypes.byref(ip), bufs[p_], bufs[p1_], bufs[q0_], bufs[q1_], flags, cnt.data_ptr(),
                self.stream_handle()), "implicit update")
            stop(p_, p1_, 0)  # converged or flat: the new iterate
            p_, p1_ = p1_, p_  # p1, p = p, p1
            if last:
                stop(p_, p1_, 1)  # exhausted: the previous iterate
                return p_, p1_, q0_, q1_
            q0_, q1_ = q1_, q0_  # q0 = q1; q1 <- the residual of the new p1
            residual(p1_, q1_, q0_)
            return p_, p1_, q0_, q1_

        graph = None
        try:
            cnt[:nb].zero_()
            stats[:nb].zero_()
            its_dev[:nb].zero_()
            counter.zero_()
            rhs_at(y, f0, t, 0)
            _native.check(lib.prml_implicit_predict(
                ctypes.byref(ip), y, f0, fu, bufs[0], bufs[1], flags, cnt.data_ptr(), self.stream_handle()),
                "implicit predict")
            residual(0, 2, None)
            residual(1, 3, 2)
            roles = (0, 1, 2, 3)
            max_it = int(s["max_iterations"])
            it, closed = 0, False
            while it < max_it:
                block_end = min(it + self.IMPLICIT_BLOCK, max_it)
                while it < block_end:
                    if block_end - it >= 2:
                        if graph is None:
                            # two iterations bring the roles back: record them
                            # once, then replay (recording runs nothing)
                            graph = torch.cuda.CUDAGraph()
                            side = self._implicit_stream
                            side.wait_stream(torch.cuda.current_stream())
                            with torch.cuda.stream(side):
                                graph.capture_begin(capture_error_mode="relaxed")
                                try:
                                    back = iteration(iteration(roles, False), False)
                                finally:
                                    graph.capture_end()
                            torch.cuda.current_stream().wait_stream(side)
                            assert back == roles
                        graph.replay()
                        it += 2
                    else:
                        it += 1
                        closed = it == max_it
                        roles = iteration(roles, closed)
                if bool(cnt[:nb, 3].all()):
                    break
            if it == max_it and not closed:
                stop(roles[0], roles[1], 1)  # the limit reached inside a replay
            its = [int(v) for v in its_dev[:nb].cpu()]
            stat = stats[:nb].cpu().numpy()
            self.secant_iterations.append(its)
            # numpy's post-loop checks (scipy.optimize.newton), instance by
            # instance in the order they stopped
            for b in sorted(range(nb), key=lambda b: (its[b], b)):
                n_fail, n_all, n_zero, rms2 = stat[b]
                if n_zero > 0:
                    if rms2 > 0:
                        msg = f"RMS of {np.sqrt(rms2):g} reached"
                        self.secant_warnings.append(msg)
                        warnings.warn(msg, RuntimeWarning, stacklevel=5)
                elif n_fail > 0:
                    all_or_some = "all" if n_fail == n_all else "some"
                    msg = f"{all_or_some} failed to converge after {s['max_iterations']:d} iterations"
                    if n_fail == n_all:
                        raise RuntimeError(msg)
                    self.secant_warnings.append(msg)
                    warnings.warn(msg, RuntimeWarning, stacklevel=5)
            _native.check(lib.prml_implicit_finish(ctypes.byref(ip), res, f0, out, self.stream_handle()),
                          "implicit finish")
        finally:
            del graph
            self.params.dirichlet, self.params.neumann = base_dir, base_neu
            self.params.batch = batch_saved
            ip.batch = self.batch

    def _run_implicit(self, y0: int, traj: int, traj_step_stride: int, work, n_steps: int, save_every: int,
                      t0: float, dt: float) -> None:
        """Steps of an implicit integrator: one secant solve per step, then
        the Jacobi solve of any LHS.Y_LAPLACIAN rows."""
        es = self.esize
        bc_bytes = int(self.params.bc_stride) * es
        nb = self.params.batch
        base_dir, base_neu = self.params.dirichlet, self.params.neumann
        cur = y0
        for s in range(n_steps):
            step = s + 1
            if step % save_every == 0:
                out = traj + (step // save_every - 1) * traj_step_stride * es
            else:
                out = _addr(work[s & 1])
            self.params.dirichlet = base_dir + 2 * s * bc_bytes
            self.params.neumann = base_neu + 2 * s * bc_bytes
            try:
                self._implicit_step(cur, out, t0 + s * dt, dt, bc_bytes, nb)
                if self.low.lap_idx:
                    self.anti_laplacian(out, 2, nb)
            finally:
                self.params.dirichlet, self.params.neumann = base_dir, base_neu
            cur = out

    def _step_kernel(self, tile):
        name, smem = self.module.gen.step_kernels[tile]
        return self.module.kernel(name, smem)

    def run(
        self,
        y0,
        traj,
        n_steps: int,
        t0: float,
        dt: float,
        save_every: int = 1,
        work=None,
        y0_bstride: Optional[int] = None,
        traj_bstride: Optional[int] = None,
        traj_step_stride: Optional[int] = None,
        batch: Optional[int] = None,
        t_offset_ptr: Optional[int] = None,
        bc_inst_slot_ptr: Optional[int] = None,
    ) -> None:
        """``n_steps`` fused steps from device state ``y0``.

        Step s (1-based) goes to ``traj`` slot ``s // save_every - 1`` when
        ``save_every`` divides s; other steps go to the two ``work`` states.
        ``y0``/``traj``/``work`` are tensors or raw device addresses; ``batch``
        runs only the first instances; ``t_offset_ptr`` is the device address
        of per-instance start-time offsets (float64).  Time-dependent
        boundary conditions: with tables preset over a longer interval
        (``preset_tables``) a run may start at any step of it, and
        ``bc_inst_slot_ptr`` (device int32 per instance, in half steps) lets
        the instances of one launch start at different times of it.
        """
        if n_steps == 0:
            return
        # per-run records: one entry per step (implicit integrators, Jacobi
        # solves), kept for the latest run only so that a reused plan does
        # not grow them without bound
        self.secant_iterations.clear()
        self.secant_warnings.clear()
        self.jacobi_iterations.clear()
        slot_base = 0
        if self.low.dynamic:
            slot_base = self._preset_slot(float(t0), float(dt), int(n_steps))
            if slot_base is None:
                if t_offset_ptr is not None or self.params.t_offset or bc_inst_slot_ptr is not None:
                    raise NotImplementedError("time-dependent boundary conditions with per-instance start times "
                                              "need tables preset over the whole interval (preset_tables)")
                self._dynamic_tables(float(t0), float(dt), int(n_steps))
                slot_base = 0
        else:
            bc_inst_slot_ptr = None  # static tables: every slot is the one table
        full = save_every == 1
        tile = self.tile or (None if self.implicit is not None else self.autotune(dt, full=full))
        self.last_tile = tile
        # the grid cap: the caller's, else the one tuned with this tile
        self.params.max_ctas = self._user_ctas or (self._tuned_ctas.get(full, 0) if self.tile is None else 0)
        self.last_ctas = self.params.max_ctas
        if save_every > 1 and work is None:
            work = self.new_state(2)
        saved = (self.params.batch, self.params.t_offset)
        if batch is not None:
            if not 1 <= batch <= self.batch:
                raise ValueError(f"batch {batch} outside 1..{self.batch}")
            self.params.batch = batch
        if t_offset_ptr is not None:
            self.params.t_offset = t_offset_ptr
        saved_tables = (self.params.dirichlet, self.params.neumann)
        if (self.implicit is not None or self.low.lap_idx) and slot_base:
            # these paths address the tables by pointer: move the base there
            off = slot_base * int(self.params.bc_stride) * self.esize
            self.params.dirichlet += off
            self.params.neumann += off
            slot_base = 0
        self.params.bc_slot0 = slot_base
        self.params.bc_inst_slot = bc_inst_slot_ptr or 0
        try:
            if self.implicit is not None:
                if t_offset_ptr is not None or self.params.t_offset:
                    raise NotImplementedError("implicit integrators take one start time per run")
                if (y0_bstride not in (None, self.inst) or traj_bstride not in (None, self.inst)):
                    raise NotImplementedError("implicit integrators need the plan's instance stride")
                self._run_implicit(_addr(y0), _addr(traj),
                                   self.params.batch * self.inst if traj_step_stride is None else traj_step_stride,
                                   work, n_steps, save_every, t0, dt)
                return
            if self.low.lap_idx:
                if t_offset_ptr is not None or self.params.t_offset:
                    raise NotImplementedError("LHS.Y_LAPLACIAN problems take one start time per run")
                self._run_jacobi(
                    tile, _addr(y0), self.inst if y0_bstride is None else y0_bstride,
                    _addr(traj), self.inst if traj_bstride is None else traj_bstride,
                    self.params.batch * self.inst if traj_step_stride is None else traj_step_stride,
                    work, n_steps, save_every, t0, dt,
                )
                return
            self._launch(
                tile, _addr(y0), self.inst if y0_bstride is None else y0_bstride,
                _addr(traj), self.inst if traj_bstride is None else traj_bstride,
                self.params.batch * self.inst if traj_step_stride is None else traj_step_stride,
                _addr(work[0]) if work is not None else 0,
                _addr(work[1]) if work is not None else 0,
                n_steps, save_every, t0, dt,
            )
        finally:
            self.params.batch, self.params.t_offset = saved
            self.params.dirichlet, self.params.neumann = saved_tables
            self.params.bc_slot0 = 0
            self.params.bc_inst_slot = 0

    def preset_tables(self, t0: float, dt: float, n_steps: int) -> None:
        """Time-dependent boundary tables for every half step of
        [t0, t0 + n_steps dt], built once; later runs with this dt that start
        on a step of that grid and end inside it use them (a base table per
        launch and optional per-instance offsets) instead of building their
        own."""
        self._dynamic_tables(float(t0), float(dt), int(n_steps))
        self._preset = (float(t0), float(dt), int(n_steps))

    def _preset_slot(self, t0: float, dt: float, n_steps: int) -> Optional[int]:
        """Half-step table of the preset grid at which a run starting at t0
        begins, or None when the run does not fit the preset tables."""
        pre = getattr(self, "_preset", None)
        if pre is None or not np.isclose(dt, pre[1], rtol=1e-12, atol=0.0):
            return None
        k = int(round((t0 - pre[0]) / (pre[1] / 2.0)))
        if k < 0 or k % 2 or not np.isclose(pre[0] + k * (pre[1] / 2.0), t0, rtol=0.0,
                                            atol=1e-9 * max(1.0, abs(t0))):
            return None
        if k + 2 * n_steps > 2 * pre[2]:
            return None
        return k

    def capture(self, y0, traj, n_steps: int, t0: float, dt: float, save_every: int = 1, work=None):
        """Records ``run(...)`` with these buffers as a CUDA graph.

        Returns the graph; ``graph.replay()`` re-issues all n_steps launches
        with one host call (the buffers must stay alive and in place).
        """
        import torch

        if self.implicit is not None:
            raise NotImplementedError("implicit integrators cannot be captured: each step's secant loop stops "
                                      "on counters the host reads")
        if self.low.lap_idx:
            raise NotImplementedError(
                "LHS.Y_LAPLACIAN problems cannot be captured: each step's Jacobi solve draws a "
                "host-side initial estimate and stops on a device-side test")
        if self.tile is None:
            self.autotune(dt, full=(save_every == 1))
        if self.low.dynamic and self._preset_slot(float(t0), float(dt), int(n_steps)) is None:
            self._dynamic_tables(float(t0), float(dt), int(n_steps))  # uploads before recording
        if save_every > 1 and work is None:
            work = self.new_state(2)
        graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(graph, stream=side):
                self.run(y0, traj, n_steps, t0, dt, save_every, work)
        torch.cuda.current_stream().wait_stream(side)
        graph._prml_keep = (y0, traj, work)
        return graph

    def _launch(self, tile, y0, y0_bstride, traj, traj_bstride, traj_step_stride, wa, wb,
                n_steps, save_every, t0, dt) -> None:
        if codegen.is_walk(tile):
            # the register-window kernels move 16 bytes per access: every
            # buffer, instance and step must start on a 16-byte boundary
            vw = 16 // self.esize
            strides = (y0_bstride, traj_bstride, traj_step_stride, self.inst)
            addrs = [a for a in (y0, traj, wa, wb) if a]
            if any(a % 16 for a in addrs) or any(s % vw for s in strides):
                raise ValueError("register-window step kernels need 16-byte aligned states and strides")
        rows, cols = self.module.gen.box(tile)
        self.params.tb_max = codegen.tile_steps(tile)
        self.params.tile_z = max(1, codegen.tile_planes(tile))
        self.params.box_planes = self.module.gen.box_depth(tile)
        _native.check(
            _native.lib().prml_fdm_run(
                self._step_kernel(tile), tile[2], tile[0], tile[1], rows, cols, self.module.gen.box_planes(tile),
                ctypes.byref(self.params), y0, y0_bstride, traj, traj_bstride, traj_step_stride,
                wa, wb, self.inst, n_steps, save_every, float(t0), float(dt), self.stream_handle(),
            ),
            "fdm run",
        )

    def rhs(self, y, f, t: float) -> None:
        """Right-hand side of every equation at (t, y) into ``f`` (device states)."""
        name, smem, tile = self.module.gen.rhs_kernel
        k = self.module.kernel(name, smem)
        rows, cols = self.module.gen.box(tile, mode=1)
        self.params.tile_z = max(1, codegen.tile_planes(tile))
        self.params.box_planes = self.module.gen.box_depth(tile, mode=1)
        _native.check(
            _native.lib().prml_fdm_rhs(
                k, tile[2], tile[0], tile[1], rows, cols, self.C, ctypes.byref(self.params),
                _addr(y), self.inst, _addr(f), self.inst, float(t), self.stream_handle(),
            ),
            "fdm rhs",
        )

    def check_status(self) -> None:
        """Raises if a kernel reported a timed-out wait since the last check."""
        flag = int(self._status.item())
        if flag:
            self._status.zero_()
            raise RuntimeError(f"a stencil kernel timed out in a bounded wait (TMA staging or grid barrier; "
                               f"status {flag})")

    # ------------------------------------------------------------------
    def _dynamic_tables(self, t0: float, dt: float, n_steps: int) -> None:
        """Boundary tables of a time-dependent problem for every half step of
        a run (table k at time t0 + k dt / 2), uploaded once per (t0, dt,
        n_steps); the kernels pick the table of each stage."""
        import torch

        key = (t0, dt, n_steps)
        if getattr(self, "_dyn_key", None) == key:
            return
        self._preset = None  # new tables replace any preset grid
        low = self.low
        n_tab = 2 * n_steps + 1
        d = np.empty((n_tab,) + low.dirichlet.shape)
        n = np.empty((n_tab,) + low.neumann.shape)
        for k in range(n_tab):
            d[k], n[k] = codegen.face_tables_at(low, t0 + k * (dt / 2.0))
        tdt = torch_dtype(self.dtype)
        self._dir_dyn = torch.tensor(d, dtype=tdt, device=self.device)
        self._neu_dyn = torch.tensor(n, dtype=tdt, device=self.device)
        self.params.dirichlet = self._dir_dyn.data_ptr()
        self.params.neumann = self._neu_dyn.data_ptr()
        self.params.bc_stride = int(np.prod(low.dirichlet.shape))
        self._dyn_key = key

    def autotune(self, dt: float, full: bool = True) -> Tuple[int, ...]:
        """Times every instantiated tile on this problem and keeps the fastest.

        ``full``: every step is stored (a full trajectory); otherwise only
        the last of several steps is.  The two patterns are tuned apart:
        temporally blocked kernels skip the stores of unsaved steps.
        """
        import torch

        if self.tile is not None:
            return self.tile
        if full in self._tuned:
            return self._tuned[full]
        key = f"{self.module.gen.key}:{self.nz}x{self.rows}x{self.ny}:b{self.batch}:{'full' if full else 'final'}:v3"
        cached = _tune_cache_load().get(key)
        if isinstance(cached, dict) and tuple(cached.get("tile", ())) in self.module.gen.step_kernels:
            self._tuned[full] = tuple(cached["tile"])
            self._tuned_ctas[full] = int(cached.get("ctas", 0))
            return self._tuned[full]
        import torch as _torch

        sms = _torch.cuda.get_device_properties(self.device).multi_processor_count
        cands = list(self.module.gen.step_kernels)
        reps = 16  # a multiple of every temporal block; best of 3 rounds per tile
        # timing launches read boundary table 0 only: a time-dependent run's
        # tables may cover fewer half steps than the timing launches take
        saved_stride, self.params.bc_stride = self.params.bc_stride, 0
        saved_ctas = self.params.max_ctas
        try:
            a = self.new_state(3)  # a[0]: start state, a[1], a[2]: work
            a.zero_()
            traj = self.new_state(reps if full else 1)
            timings = []  # (ms per `reps` steps, tile, grid cap, timing function)
            for tile in cands:
                k = self._step_kernel(tile)
                occ = ctypes.c_int()
                _native.check(_native.lib().prml_kernel_occupancy(k, tile[2], ctypes.byref(occ)), "occupancy")
                if occ.value < 1:
                    continue
                # grid density: every resident CTA (one round of tiles), or
                # fewer CTAs per SM that each walk several tiles and stage the
                # next tile while computing the current one
                caps = [0] + [sms * c for c in (2, 4, 8) if c < occ.value]

                def go(n, tile=tile):
                    self._launch(
                        tile, a[0].data_ptr(), self.inst, traj[0].data_ptr(), self.inst,
                        self.batch * self.inst, a[1].data_ptr(), a[2].data_ptr(), n, 1 if full else n, 0.0, dt,
                    )

                def timed(rounds, go=go):
                    # rounds of `reps` steps each (the trajectory holds reps slots)
                    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    start.record()
                    for _ in range(rounds):
                        go(reps)
                    stop.record()
                    stop.synchronize()
                    return start.elapsed_time(stop)

                for cap in caps:
                    self.params.max_ctas = cap
                    go(2)
                    timings.append((min(timed(1) for _ in range(3)), tile, cap, timed))
            # the three fastest again with timings of at least ~2 ms each, so
            # that launch jitter does not pick the tile of a fast kernel
            best, best_caps, best_t = cands[0], 0, float("inf")
            for ms1, tile, cap, timed in sorted(timings, key=lambda e: e[0])[:3]:
                self.params.max_ctas = cap
                rounds = max(1, min(16, int(2.0 / max(ms1, 1e-3))))
                ms = min(timed(rounds) for _ in range(3)) / rounds
                if ms < best_t:
                    best, best_caps, best_t = tile, cap, ms
        finally:
            self.params.bc_stride = saved_stride
            self.params.max_ctas = saved_ctas
        self._tuned[full] = best
        self._tuned_ctas[full] = best_caps
        _tune_cache_store(key, {"tile": list(best), "ctas": best_caps})
        return best


class MultiRun:
    """Every step of several groups of batched solves in ONE cooperative
    launch (``prml_multi_launch``, kernels ``prml_multi_*`` of a module built
    with ``multi=True``).

    Each group is a plan (its mesh, tables and batch), the device state its
    first step reads, a slotted output buffer, its step count, start time
    and step size.  Round r of the launch is step r of every group with more
    than r steps; the tiles of a round are spread over the whole grid and a
    grid barrier separates the rounds.  ``ping_pong`` groups keep only the
    final state (two slots); the others store every step in its own slot (a
    trajectory).  All groups must share the plans' generated module (same
    equation, boundary kinds and precision); the tile is tuned over the
    ensemble as a whole.  ``launch()`` issues the barrier reset and the
    kernel on the current stream (both can be recorded in a CUDA graph).
    """

    def __init__(self, groups, tile=None, max_ctas: int = 0):
        import torch

        if not groups or len(groups) > _native.MULTI_MAX_GROUPS:
            raise ValueError(f"a multi-round launch takes 1 to {_native.MULTI_MAX_GROUPS} groups")
        plan0 = groups[0]["plan"]
        for g in groups:
            if g["plan"].module is not plan0.module:
                raise ValueError("the groups of a multi-round launch must share one generated module")
            if g["plan"].implicit is not None or g["plan"].low.lap_idx:
                raise NotImplementedError("multi-round launches take explicit steps without Jacobi rows")
        if not plan0.module.gen.multi_kernels:
            raise NotImplementedError("the plans' module has no multi-round kernels (build them with multi=True)")
        self.groups = groups
        self.plan0 = plan0
        self.max_ctas = int(max_ctas)
        lib = _native.lib()
        self._lib = lib
        nbytes = int(lib.prml_multi_desc_bytes(len(groups)))
        dev = plan0.device
        self._desc = {}
        self._desc_bytes = nbytes
        self._barrier = torch.zeros(1, dtype=torch.int64, device=dev)
        self.n_rounds = max(int(g["n_steps"]) for g in groups)
        for g in groups:
            p = g["plan"]
            if p.low.dynamic:
                p._dynamic_tables(float(g["t0"]), float(g["dt"]), int(g["n_steps"]))
        self.tile = tuple(tile) if tile is not None else self.autotune()
        if self.tile not in plan0.module.gen.multi_kernels:
            raise ValueError(f"tile {self.tile} has no multi-round kernel in this module")

    def _groups_array(self, tile):
        arr = (_native.MultiGroup * len(self.groups))()
        tiles = 0
        for k, g in enumerate(self.groups):
            plan = g["plan"]
            mg = arr[k]
            mg.p = plan.params
            mg.p.batch = int(g.get("batch", plan.batch))
            mg.p.in_bstride = mg.p.out_bstride = plan.inst
            mg.p.t_offset = 0
            mg.p.dt = float(g["dt"])
            mg.p.dt_f = float(g["dt"])
            mg.p.tb_max = 1
            mg.p.tile_z = 1
            mg.p.box_planes = 1
            mg.p.status = self.plan0._status.data_ptr()
            mg.first = _addr(g["first"])
            mg.main = _addr(g["main"])
            mg.slot_stride = int(g.get("slot_stride", plan.batch * plan.inst))
            mg.t0 = float(g["t0"])
            mg.n_steps = int(g["n_steps"])
            mg.ping_pong = 1 if g.get("ping_pong", True) else 0
            tiles += mg.p.batch * (-(-plan.ny // tile[1])) * (-(-plan.nx // tile[0]))
        return arr, tiles

    def _prepare(self, tile):
        import torch

        entry = self._desc.get(tile)
        if entry is not None:
            return entry
        gen = self.plan0.module.gen
        rows, cols = gen.box(tile)
        arr, tiles = self._groups_array(tile)
        desc = torch.empty(self._desc_bytes, dtype=torch.uint8, device=self.plan0.device)
        _native.check(self._lib.prml_multi_prepare(ctypes.byref(arr), len(self.groups), tile[0], tile[1], rows, cols,
                                                   gen.box_planes(tile), desc.data_ptr(), desc.numel()),
                      "multi-round prepare")
        name, smem = gen.multi_kernels[tile]
        kernel = self.plan0.module.kernel(name, smem)
        entry = (desc, tiles, kernel, arr)
        self._desc[tile] = entry
        return entry

    def launch(self, tile=None) -> None:
        tile = self.tile if tile is None else tile
        desc, tiles, kernel, _ = self._prepare(tile)
        _native.check(self._lib.prml_multi_launch(kernel, tile[2], desc.data_ptr(), len(self.groups), self.n_rounds,
                                                  tiles, self._barrier.data_ptr(), self.plan0._status.data_ptr(),
                                                  self.max_ctas, StencilPlan.stream_handle()),
                      "multi-round launch")

    def autotune(self):
        """Times every multi-round tile on the actual groups and keeps the fastest."""
        import torch

        best, best_t = None, float("inf")
        for tile in self.plan0.module.gen.multi_kernels:
            _, _, kernel, _ = self._prepare(tile)
            occ = ctypes.c_int()
            _native.check(self._lib.prml_kernel_occupancy(kernel, tile[2], ctypes.byref(occ)), "occupancy")
            if occ.value < 1:  # registers or shared memory of this tile exceed an SM
                continue
            self.launch(tile)
            ms = float("inf")
            for _ in range(2):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                self.launch(tile)
                b.record()
                b.synchronize()
                ms = min(ms, a.elapsed_time(b))
            if ms < best_t:
                best, best_t = tile, ms
        self.plan0.check_status()
        if best is None:
            raise NotImplementedError("no multi-round tile fits on an SM for this system")
        return best

    def check_status(self) -> None:
        self.plan0.check_status()
