"""Build and ctypes binding of the C-ABI library ``libprml_gb300.so``.

The library is compiled in-tree for sm_103a by ``build()`` (one nvcc
process per source file, in parallel, then one link) and loaded with
``ctypes``; every call goes through the C ABI
declared in ``include/pararealml_gb300.h``.  There is no CPU fallback: if the
library or a CUDA device is missing, ``lib()`` raises.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from typing import Optional

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC_DIR = os.path.join(PKG_DIR, "csrc")
INCLUDE_DIR = os.path.join(REPO_DIR, "include")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libprml_gb300.so")
JIT_CACHE_DIR = os.path.join(PKG_DIR, "_jit")
ARCH = "sm_103a"
SOURCES = ("prml_core.cpp", "prml_parareal.cu", "prml_layout.cu", "prml_cnn.cu", "prml_cnn_tc.cu", "prml_jacobi.cu",
           "prml_implicit.cu", "prml_measure.cu")

PRML_OK, PRML_ERR_ARG, PRML_ERR_COMPILE, PRML_ERR_CUDA, PRML_ERR_UNSUPPORTED = 0, 1, 2, 3, 4
PRML_ERR_CONVERGENCE = 5

_lock = threading.Lock()
_lib: Optional[ctypes.CDLL] = None


def nvcc_path() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC_DIR, f) for f in os.listdir(CSRC_DIR)]
    deps += [os.path.join(INCLUDE_DIR, f) for f in os.listdir(INCLUDE_DIR)]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False) -> str:
    """Compiles libprml_gb300.so for sm_103a: every source file to an object
    in its own nvcc process (all at once), then one shared-library link."""
    from concurrent.futures import ThreadPoolExecutor

    os.makedirs(LIB_DIR, exist_ok=True)
    if not force and not _stale():
        return LIB_PATH
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    tag = f"{os.getpid()}"
    flags = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo",
             f"-I{INCLUDE_DIR}", f"-I{CSRC_DIR}"]
    objs = [os.path.join(LIB_DIR, f"{os.path.splitext(src)[0]}.{tag}.o") for src in SOURCES]

    def compile_one(k: int) -> None:
        subprocess.run([nvcc_path(), *flags, "-c", os.path.join(CSRC_DIR, SOURCES[k]), "-o", objs[k]], check=True)

    tmp = LIB_PATH + f".tmp{tag}"
    try:
        with ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
            list(pool.map(compile_one, range(len(SOURCES))))
        subprocess.run([nvcc_path(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", tmp,
                        "-cudart", "shared", f"-L{os.path.join(cuda, 'lib64')}", "-lnvrtc", "-ldl",
                        f"-Xlinker=-rpath,{os.path.join(cuda, 'lib64')}"], check=True)
        os.replace(tmp, LIB_PATH)
    finally:
        for o in objs + [tmp]:
            if os.path.exists(o):
                os.remove(o)
    return LIB_PATH


_c_int, _c_ll, _c_d, _p = ctypes.c_int, ctypes.c_longlong, ctypes.c_double, ctypes.c_void_p


def _declare(lib: ctypes.CDLL) -> None:
    sig = {
        "prml_last_error": (ctypes.c_char_p, []),
        "prml_abi_version": (_c_int, []),
        "prml_step_params_size": (_c_int, []),
        "prml_jit_compile": (
            _c_int,
            [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _c_ll],
        ),
        "prml_module_load": (_c_int, [ctypes.c_char_p, ctypes.POINTER(_p)]),
        "prml_module_unload": (_c_int, [_p]),
        "prml_module_kernel": (_c_int, [_p, ctypes.c_char_p, _c_int, ctypes.POINTER(_p)]),
        "prml_kernel_free": (_c_int, [_p]),
        "prml_kernel_occupancy": (_c_int, [_p, _c_int, ctypes.POINTER(_c_int)]),
        "prml_fdm_run": (
            _c_int,
            [_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _p, _p, _c_ll, _p, _c_ll, _c_ll, _p, _p, _c_ll, _c_ll, _c_int, _c_d, _c_d, _p],
        ),
        "prml_fdm_rhs": (_c_int, [_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _p, _p, _c_ll, _p, _c_ll, _c_d, _p]),
        "prml_set_step_overlap": (_c_int, [_c_int]),
        "prml_pack": (_c_int, [_p, _p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_ll, _c_ll, _c_int, _p]),
        "prml_unpack": (_c_int, [_p, _c_int, _p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_ll, _c_ll, _c_int, _p]),
        "prml_pr_cast": (_c_int, [_p, _p, _c_int, _c_ll, _c_ll, _p]),
        "prml_pr_correct": (_c_int, [_p, _c_int, _p, _p, _c_ll, _c_ll, _p, _c_int, _c_ll, _p]),
        "prml_pr_advance": (_c_int, [_p, _c_int, _p, _p, _p, _p, _c_ll, _c_ll, _p, _c_int, _c_ll, _p]),
        "prml_pr_copy": (_c_int, [_p, _p, _c_ll, _c_ll, _p, _c_int, _p]),
        "prml_pr_end_delta": (_c_int, [_p, _p, _c_int, _p, _c_ll, _c_ll, _p]),
        "prml_pr_norm_scratch_elems": (_c_ll, [_c_int, _c_int, _c_int, _c_int]),
        "prml_pr_update_norm": (
            _c_int,
            [_p, _p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _p, _p, _p],
        ),
        "prml_cnn_in_fwd": (_c_int, [_p, _c_int, _c_int, _p, _p, _p, _p, _c_int, _c_int, _c_int, _p]),
        "prml_cnn_mid_fwd": (_c_int, [_p, _p, _p, _p, _c_int, _c_int, _c_int, _p]),
        "prml_cnn_out_fwd": (_c_int, [_p, _p, _p, _p, _p, _p, _c_int, _c_int, _c_int, _c_int, _c_int, _p]),
        "prml_cnn_out_bwd": (_c_int, [_p, _p, _p, _p, _p, _p, _p, _c_int, _p, _c_int, _c_int, _c_int, _p]),
        "prml_cnn_mid_dgrad": (_c_int, [_p, _p, _p, _p, _c_int, _c_int, _c_int, _p]),
        "prml_cnn_wgrad_scratch_elems": (_c_ll, [_c_int]),
        "prml_cnn_mid_wgrad": (_c_int, [_p, _p, _p, _p, _c_int, _p, _c_int, _c_int, _c_int, _p]),
        "prml_cnn_thin_scratch_elems": (_c_ll, [_c_int]),
        "prml_cnn_in_wgrad": (_c_int, [_p, _p, _c_int, _c_int, _p, _p, _p, _c_int, _p, _c_int, _c_int, _c_int, _p]),
        "prml_cnn_mse": (_c_int, [_p, _p, _c_int, _c_int, _c_int, _c_int, _c_int, _p, _p, _c_int, _p]),
        "prml_cnn_adam": (_c_int, [_p, _p, _p, _p, _c_ll, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, _c_int, _p]),
        "prml_cnn_pack_mid": (_c_int, [_p, _p, _p, _p]),
        "prml_cnn_set_tensor_path": (_c_int, [_c_int]),
        "prml_cnn_status": (_c_int, []),
        "prml_pr_update_norm_noalloc": (
            _c_int,
            [_p, _p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _p, _p],
        ),
        "prml_jacobi_params_size": (_c_int, []),
        "prml_jacobi_scratch_bytes": (_c_ll, [_p]),
        "prml_anti_laplacian": (_c_int, [_p, _p, _p, _p, _c_ll, ctypes.POINTER(_c_ll), _p]),
        "prml_implicit_params_size": (_c_int, []),
        "prml_implicit_predict": (_c_int, [_p, _p, _p, _p, _p, _p, _p, _p, _p]),
        "prml_implicit_residual": (_c_int, [_p, _p, _p, _p, _p, _p, _p, _p, _p]),
        "prml_implicit_update": (_c_int, [_p, _p, _p, _p, _p, _p, _p, _p]),
        "prml_implicit_status": (_c_int, [_p, _p, _p, _p, _p, _p]),
        "prml_implicit_stop": (_c_int, [_p, _p, _p, _p, _p, _p, _c_int, _p, _p, _p, _p]),
        "prml_implicit_finish": (_c_int, [_p, _p, _p, _p, _p]),
        "prml_measure_fp64_fma": (_c_int, [ctypes.POINTER(_c_d), _p]),
        "prml_gaussian_states": (_c_int, [_p, _c_ll, _c_int, _p, _c_int, _c_int, _p, _p]),
        "prml_multi_group_size": (_c_int, []),
        "prml_multi_desc_bytes": (_c_ll, [_c_int]),
        "prml_multi_prepare": (_c_int, [_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _p, _c_ll]),
        "prml_multi_launch": (_c_int, [_p, _c_int, _p, _c_int, _c_int, _c_ll, _p, _p, _c_int, _p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def exported_symbols() -> list:
    """Names the C header declares (for the export check)."""
    return [
        "prml_last_error",
        "prml_abi_version",
        "prml_step_params_size",
        "prml_jit_compile",
        "prml_module_load",
        "prml_module_unload",
        "prml_module_kernel",
        "prml_kernel_free",
        "prml_kernel_occupancy",
        "prml_fdm_run",
        "prml_fdm_rhs",
        "prml_set_step_overlap",
        "prml_pack",
        "prml_unpack",
        "prml_pr_cast",
        "prml_pr_correct",
        "prml_pr_advance",
        "prml_pr_copy",
        "prml_pr_end_delta",
        "prml_pr_norm_scratch_elems",
        "prml_pr_update_norm",
        "prml_pr_update_norm_noalloc",
        "prml_cnn_in_fwd",
        "prml_cnn_mid_fwd",
        "prml_cnn_out_fwd",
        "prml_cnn_out_bwd",
        "prml_cnn_mid_dgrad",
        "prml_cnn_wgrad_scratch_elems",
        "prml_cnn_mid_wgrad",
        "prml_cnn_thin_scratch_elems",
        "prml_cnn_in_wgrad",
        "prml_cnn_mse",
        "prml_cnn_adam",
        "prml_cnn_pack_mid",
        "prml_cnn_set_tensor_path",
        "prml_cnn_status",
        "prml_jacobi_params_size",
        "prml_jacobi_scratch_bytes",
        "prml_anti_laplacian",
        "prml_implicit_params_size",
        "prml_implicit_predict",
        "prml_implicit_residual",
        "prml_implicit_update",
        "prml_implicit_status",
        "prml_implicit_stop",
        "prml_implicit_finish",
        "prml_measure_fp64_fma",
        "prml_gaussian_states",
        "prml_multi_group_size",
        "prml_multi_desc_bytes",
        "prml_multi_prepare",
        "prml_multi_launch",
    ]


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads the library (no device needed) and declares its signatures."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise RuntimeError(
                    f"{path} is missing: run pararealml_gb300._native.build() first"
                )
            lib = ctypes.CDLL(path)
            _declare(lib)
            _lib = lib
        return _lib


def lib() -> ctypes.CDLL:
    """The library, for compute calls: requires a CUDA device."""
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("pararealml_gb300 needs a CUDA device; no CPU fallback exists")
    torch.cuda.init()
    return load_library()


class PrmlError(RuntimeError):
    pass


class ConvergenceError(PrmlError):
    """An iterative solve (the Jacobi anti-Laplacian) hit its iteration cap."""


def check(rc: int, what: str = "") -> None:
    if rc == PRML_OK:
        return
    msg = load_library().prml_last_error().decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if rc == PRML_ERR_ARG:
        raise ValueError(text)
    if rc == PRML_ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    if rc == PRML_ERR_CONVERGENCE:
        raise ConvergenceError(text)
    raise PrmlError(text)


TB_MAX = 8  # PRML_TB_MAX: most time steps of one temporally blocked launch


class StepParams(ctypes.Structure):
    """Mirror of ``prml_step_params`` (include/prml_params.h)."""

    _fields_ = [
        ("in_", _p),
        ("out", _p),
        ("in_bstride", _c_ll),
        ("out_bstride", _c_ll),
        ("cstride", _c_ll),
        ("pitch", _c_int),
        ("nx", _c_int),
        ("ny", _c_int),
        ("batch", _c_int),
        ("face_len", _c_int),
        ("elem_bytes", _c_int),
        ("t", _c_d),
        ("dt", _c_d),
        ("t_offset", _p),
        ("dirichlet", _p),
        ("neumann", _p),
        ("coord0", _p),
        ("coord1", _p),
        ("inv_2dx0", _c_d),
        ("inv_2dx1", _c_d),
        ("inv_dxx0", _c_d),
        ("inv_dxx1", _c_d),
        ("two_dx0", _c_d),
        ("two_dx1", _c_d),
        ("in_slot", _c_int),
        ("max_ctas", _c_int),
        ("status", _p),
        ("tb_max", _c_int),
        ("tb_steps", _c_int),
        ("tb_bstride", _c_ll),
        ("tb_out", _p * (TB_MAX - 1)),
        ("dt_f", ctypes.c_float),
        ("inv_2dx0_f", ctypes.c_float),
        ("inv_2dx1_f", ctypes.c_float),
        ("inv_dxx0_f", ctypes.c_float),
        ("inv_dxx1_f", ctypes.c_float),
        ("two_dx0_f", ctypes.c_float),
        ("two_dx1_f", ctypes.c_float),
        ("coord0_f", _p),
        ("coord1_f", _p),
        ("bc_stride", _c_ll),
        ("bc_slot0", _c_int),
        ("nz", _c_int),
        ("tile_z", _c_int),
        ("box_planes", _c_int),
        ("inv_2dx2", _c_d),
        ("inv_dxx2", _c_d),
        ("two_dx2", _c_d),
        ("inv_2dx2_f", ctypes.c_float),
        ("inv_dxx2_f", ctypes.c_float),
        ("two_dx2_f", ctypes.c_float),
        ("pad3", _c_int),
        ("coord2", _p),
        ("coord2_f", _p),
        ("dxx0", _c_d),
        ("dxx1", _c_d),
        ("dxx2", _c_d),
        ("wait_limit_ns", ctypes.c_ulonglong),
        ("wait_probe", _c_int),
        ("pad4", _c_int),
        ("bc_inst_slot", _p),
    ]


MULTI_MAX_GROUPS = 8  # PRML_MULTI_MAX_GROUPS


class MultiGroup(ctypes.Structure):
    """Mirror of ``prml_multi_group`` (include/prml_params.h)."""

    _fields_ = [
        ("p", StepParams),
        ("first", _p),
        ("main", _p),
        ("slot_stride", _c_ll),
        ("t0", _c_d),
        ("n_steps", _c_int),
        ("ping_pong", _c_int),
        ("tiles_x", _c_int),
        ("tiles_y", _c_int),
    ]


JACOBI_MAX_BATCH = 64  # PRML_JACOBI_MAX_BATCH


class JacobiParams(ctypes.Structure):
    """Mirror of ``prml_jacobi_params`` (include/pararealml_gb300.h)."""

    _fields_ = [
        ("n", _c_int * 3),
        ("first_axis", _c_int),
        ("coord_system", _c_int),
        ("comps", _c_int),
        ("n_lap", _c_int),
        ("lap_comp", _c_int * 16),
        ("elem_bytes", _c_int),
        ("batch", _c_int),
        ("pitch", _c_int),
        ("face_len", _c_int),
        ("face_base", _c_int),
        ("cstride", _c_ll),
        ("inst", _c_ll),
        ("dir_mask", ctypes.c_ulonglong),
        ("neu_mask", ctypes.c_ulonglong),
        ("dirichlet", _p),
        ("neumann", _p),
        ("inv_dxx", _c_d * 3),
        ("two_dx", _c_d * 3),
        ("coef", _p),
        ("tol", _c_d),
        ("max_iterations", _c_ll),
    ]


class ImplicitParams(ctypes.Structure):
    """Mirror of ``prml_implicit_params`` (include/pararealml_gb300.h)."""

    _fields_ = [
        ("n", _c_int * 3),
        ("first_axis", _c_int),
        ("comps", _c_int),
        ("batch", _c_int),
        ("pitch", _c_int),
        ("face_len", _c_int),
        ("face_base", _c_int),
        ("crank_nicolson", _c_int),
        ("cstride", _c_ll),
        ("inst", _c_ll),
        ("d_mask", ctypes.c_ulonglong),
        ("dir_mask", ctypes.c_ulonglong),
        ("dirichlet", _p),
        ("dt", _c_d),
        ("a", _c_d),
        ("tol", _c_d),
        ("dx", _c_d),
    ]


def jit_module(source: str, key: str, extra_options: str = "") -> str:
    """Compiles a generated module to a cached cubin and returns its path."""
    os.makedirs(JIT_CACHE_DIR, exist_ok=True)
    path = os.path.join(JIT_CACHE_DIR, f"{key}.cubin")
    if os.path.exists(path):
        return path
    log = ctypes.create_string_buffer(1 << 16)
    rc = load_library().prml_jit_compile(
        source.encode(),
        f"{CSRC_DIR};{INCLUDE_DIR}".encode(),
        ARCH.encode(),
        extra_options.encode(),
        path.encode(),
        log,
        len(log),
    )
    check(rc, "run-time compilation of a generated stencil module")
    return path


def round_up(n: int, m: int) -> int:
    return (n + m - 1) // m * m


def ptr(t) -> int:
    """Device address of a torch tensor (or 0 for None)."""
    return 0 if t is None else int(t.data_ptr())


def as_f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)
