"""The C-ABI library builds, loads without a GPU and exports its header."""

import ctypes
import os
import re

import pytest

from pararealml_gb300 import _native


def _declared_functions():
    names = set()
    for fn in os.listdir(_native.INCLUDE_DIR):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(_native.INCLUDE_DIR, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(prml_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_builds_and_exports_every_declared_symbol():
    _native.build()
    lib = _native.load_library()
    declared = _declared_functions()
    assert declared, "no declarations found"
    assert declared == set(_native.exported_symbols())
    for name in declared:
        assert hasattr(lib, name), name


def test_abi_version_and_params_layout():
    lib = _native.load_library()
    assert lib.prml_abi_version() == 1
    assert lib.prml_step_params_size() == ctypes.sizeof(_native.StepParams)
    assert lib.prml_jacobi_params_size() == ctypes.sizeof(_native.JacobiParams)
    assert lib.prml_implicit_params_size() == ctypes.sizeof(_native.ImplicitParams)
    assert lib.prml_multi_group_size() == ctypes.sizeof(_native.MultiGroup)


def test_implicit_argument_errors_without_a_device():
    """The reference's ValueErrors of the implicit integrators
    (numerical_integrator.py:146-152, 238-239) come back as PRML_ERR_ARG
    before any device call."""
    lib = _native.load_library()
    ip = _native.ImplicitParams()
    ip.n[0], ip.n[1], ip.n[2] = 1, 5, 6
    ip.first_axis, ip.comps, ip.batch, ip.pitch = 1, 1, 1, 32
    ip.cstride, ip.inst = 5 * 32, 5 * 32
    ip.a, ip.tol, ip.dx = 1.5, 1e-8, 1e-5
    assert lib.prml_implicit_finish(ctypes.byref(ip), 8, 8, 8, None) == _native.PRML_ERR_ARG
    assert b"between 0 and 1" in lib.prml_last_error()
    ip.a, ip.tol = 0.5, -1.0
    assert lib.prml_implicit_finish(ctypes.byref(ip), 8, 8, 8, None) == _native.PRML_ERR_ARG
    assert b"non-negative" in lib.prml_last_error()
    ip.tol = 1e-8
    assert lib.prml_implicit_update(ctypes.byref(ip), None, 8, 8, 8, 8, 8, None) == _native.PRML_ERR_ARG


def test_anti_laplacian_argument_errors_without_a_device():
    """The reference's ValueError for meshes with fewer than 3 points per
    axis (numerical_differentiator.py:1103-1106) and the parameter checks
    come back as PRML_ERR_ARG before any device call."""
    lib = _native.load_library()
    jp = _native.JacobiParams()
    jp.n[0], jp.n[1], jp.n[2] = 1, 5, 2
    jp.first_axis, jp.comps, jp.n_lap, jp.elem_bytes, jp.batch = 1, 2, 1, 8, 1
    jp.lap_comp[0] = 1
    jp.coef = jp.dirichlet = jp.neumann = 8
    jp.tol, jp.max_iterations = 1e-3, 10
    rc = lib.prml_anti_laplacian(ctypes.byref(jp), 8, 8, 8, 1 << 20, None, None)
    assert rc == _native.PRML_ERR_ARG
    assert b"at least 3 points" in lib.prml_last_error()
    jp.n[2] = 4
    jp.batch = _native.JACOBI_MAX_BATCH + 1
    assert lib.prml_anti_laplacian(ctypes.byref(jp), 8, 8, 8, 1 << 20, None, None) == _native.PRML_ERR_ARG
    jp.batch = 1
    jp.lap_comp[0] = 2  # not a component of a 2-component state
    assert lib.prml_anti_laplacian(ctypes.byref(jp), 8, 8, 8, 1 << 20, None, None) == _native.PRML_ERR_ARG
    assert lib.prml_jacobi_scratch_bytes(ctypes.byref(jp)) == -1


def test_errors_are_reported_without_a_device():
    lib = _native.load_library()
    rc = lib.prml_fdm_run(None, 256, 32, 32, 34, 40, 1, None, None, 0, None, 0, 0, None, None, 0, 1, 1, 0.0, 0.1, None)
    assert rc == _native.PRML_ERR_ARG
    assert b"null kernel" in lib.prml_last_error()
    rc = lib.prml_pr_update_norm(None, None, 1, 1, 1, 1, 1, 1, 1, None, None, None)
    assert rc == _native.PRML_ERR_ARG


def test_every_call_site_passes_the_declared_argument_count():
    """Static check of the Python side of the ABI: each ``.prml_*(...)``
    call in the package passes as many arguments as the C declaration."""
    import ast

    lib = _native.load_library()
    pkg = os.path.dirname(_native.__file__)
    checked = 0
    for root, _, files in os.walk(pkg):
        for fn in files:
            if not fn.endswith(".py"):
                continue
            tree = ast.parse(open(os.path.join(root, fn)).read())
            for node in ast.walk(tree):
                if isinstance(node, ast.Call) and isinstance(node.func, ast.Attribute) and node.func.attr.startswith("prml_"):
                    want = len(getattr(lib, node.func.attr).argtypes)
                    assert len(node.args) == want, f"{fn}:{node.lineno} {node.func.attr} passes {len(node.args)} of {want}"
                    checked += 1
    assert checked > 10


def test_c_host_compiles_against_the_header(tmp_path):
    """The C host of tests/c_host (a non-Python caller of the C ABI) builds
    with gcc -Wall -Werror against include/ and links to the library."""
    import shutil

    if shutil.which("gcc") is None:
        pytest.skip("gcc is not installed")
    from test_gpu_c_host import build_c_host

    _native.build()
    assert os.path.exists(build_c_host(str(tmp_path)))
