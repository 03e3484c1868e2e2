"""A C host drives FDM steps through the C ABI alone (needs a GB300).

``tests/c_host/prml_c_host.c`` is compiled with gcc against
``include/pararealml_gb300.h`` and the in-tree library, given a generated
module (cubin) and a plan's parameter block, tables and initial state as
files, and runs the steps with ``prml_pack`` / ``prml_fdm_run`` /
``prml_unpack``.  Its result must equal the Python operator's bit for bit
(same kernel, same parameters, float64).
"""

import os
import subprocess

import numpy as np
import pytest

import pararealml_gb300 as ns
import problems
from pararealml_gb300 import _native
from pararealml_gb300.operators import fdm

HERE = os.path.dirname(os.path.abspath(__file__))


def build_c_host(out_dir: str) -> str:
    """gcc the C host against the header and the in-tree library."""
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = os.path.join(out_dir, "prml_c_host")
    subprocess.run(
        ["gcc", "-O2", "-std=c11", "-Wall", "-Werror", f"-I{_native.INCLUDE_DIR}", f"-I{os.path.join(cuda, 'include')}",
         os.path.join(HERE, "c_host", "prml_c_host.c"), "-o", exe, f"-L{_native.LIB_DIR}", "-lprml_gb300",
         f"-L{os.path.join(cuda, 'lib64')}", "-lcudart", f"-Wl,-rpath,{_native.LIB_DIR}",
         f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"],
        check=True,
    )
    return exe


@pytest.mark.gpu
def test_c_host_steps_equal_the_python_operator(tmp_path):
    _native.build()
    exe = build_c_host(str(tmp_path))
    ivp = problems.cahn_hilliard_2d(ns, n=60, length=15.0, t_end=0.012)
    tile = (16, 32, 128)
    op = fdm.FDMOperator(fdm.RK4(), fdm.ThreePointCentralDifferenceMethod(), 0.001, trajectory="final", tile=tile)
    want = op.solve(ivp).discrete_y()[-1]
    plan = op.plan(ivp.constrained_problem, 1)
    gen = plan.module.gen
    name, smem = gen.step_kernels[tile]
    rows, cols = gen.box(tile)
    cubin = _native.jit_module(gen.source, gen.key, "--fmad=false")
    run = tmp_path / "run"
    run.mkdir()
    (run / "run.txt").write_text(f"{cubin} {name} {smem} {tile[2]} {tile[0]} {tile[1]} {rows} {cols} {plan.C} 12 0.001\n")
    (run / "params.bin").write_bytes(bytes(plan.params))
    for fname, t in (("dir.bin", plan._dir), ("neu.bin", plan._neu), ("c0.bin", plan._c0), ("c1.bin", plan._c1),
                     ("cz.bin", plan._cz), ("c0f.bin", plan._c0f), ("c1f.bin", plan._c1f), ("czf.bin", plan._czf)):
        (run / fname).write_bytes(t.cpu().numpy().tobytes())
    (run / "y0.bin").write_bytes(np.ascontiguousarray(ivp.initial_condition.discrete_y_0(True), dtype=np.float64)
                                 .tobytes())
    res = subprocess.run([exe, str(run)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    got = np.fromfile(run / "out.bin", dtype=np.float64).reshape(want.shape)
    assert np.array_equal(got, want)
