"""Import shim for the reference PararealML package (test infrastructure only).

The reference (ViktorC/PararealML) is pure Python.  In this container three of
its imports fail, and this module patches each one so that the UNMODIFIED
reference can be imported read-only:

1. ``matplotlib`` is absent (``pararealml/plot.py:6-18`` imports it at module
   load, pulled in by ``pararealml/__init__.py`` and ``pararealml/solution.py:11``).
   Stub modules whose attributes resolve to further stubs are installed.
2. ``mpi4py`` is absent (``pararealml/operators/parareal/parareal_operator.py:5``).
   A fake ``mpi4py.MPI`` is installed with a thread-per-rank ``COMM_WORLD``
   (``rank`` is thread-local, ``Allgather`` and ``barrier`` go through a
   ``threading.Barrier`` and a shared buffer), which is enough to run the
   reference's ``PararealOperator.solve`` with several ranks as threads.
3. numpy 2.x removed ``np.product`` (used at ``pararealml/mesh.py:384,420``);
   it is aliased to ``np.prod``.

Nothing here is shipped or imported by the product package; only the golden
fixture generator and CPU cross-check tests use it, and only where the
reference source tree is present.
"""

from __future__ import annotations

import os
import sys
import threading
import types
from typing import Callable, List, Optional

import numpy as np

# the reference source tree: PRML_REFERENCE_ROOT, else a `reference`
# directory beside this repository
REFERENCE_ROOT = os.environ.get(
    "PRML_REFERENCE_ROOT",
    os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "reference"),
)


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_ROOT, "pararealml", "__init__.py"))


class _StubModule(types.ModuleType):
    def __getattr__(self, name: str):
        if name.startswith("__"):
            raise AttributeError(name)
        child = _StubModule(f"{self.__name__}.{name}")
        setattr(self, name, child)
        return child

    def __call__(self, *args, **kwargs):
        return _StubModule(f"{self.__name__}()")


class _FakeComm:
    """Thread-per-rank stand-in for ``MPI.COMM_WORLD``."""

    def __init__(self):
        self._local = threading.local()
        self.size = 1
        self._barrier: Optional[threading.Barrier] = None
        self._slots: List[Optional[np.ndarray]] = []

    @property
    def rank(self) -> int:
        return getattr(self._local, "rank", 0)

    def _set(self, size: int):
        self.size = size
        self._barrier = threading.Barrier(size) if size > 1 else None
        self._slots = [None] * size

    def barrier(self):
        if self._barrier is not None:
            self._barrier.wait()

    def Allgather(self, send, recv):  # noqa: N802 (mpi4py spelling)
        send_buf = send[0] if isinstance(send, (list, tuple)) else send
        recv_buf = recv[0] if isinstance(recv, (list, tuple)) else recv
        if self.size == 1:
            recv_buf.reshape(-1)[:] = np.asarray(send_buf).reshape(-1)
            return
        self._slots[self.rank] = np.array(send_buf, copy=True)
        self.barrier()
        flat = recv_buf.reshape(self.size, -1)
        for r in range(self.size):
            flat[r] = self._slots[r].reshape(-1)
        self.barrier()


_COMM = _FakeComm()


def _install_stubs():
    if not hasattr(np, "product"):
        np.product = np.prod  # type: ignore[attr-defined]
    if "matplotlib" not in sys.modules or not hasattr(sys.modules["matplotlib"], "__file__"):
        for name in [
            "matplotlib",
            "matplotlib.pyplot",
            "matplotlib.cm",
            "matplotlib.animation",
            "matplotlib.collections",
            "matplotlib.colors",
            "matplotlib.contour",
            "matplotlib.figure",
            "matplotlib.lines",
            "matplotlib.quiver",
            "matplotlib.streamplot",
            "mpl_toolkits",
            "mpl_toolkits.mplot3d",
            "mpl_toolkits.mplot3d.art3d",
        ]:
            sys.modules.setdefault(name, _StubModule(name))
    if "mpi4py" not in sys.modules:
        mpi4py = types.ModuleType("mpi4py")
        mpi = types.ModuleType("mpi4py.MPI")
        mpi.COMM_WORLD = _COMM
        mpi.DOUBLE = "double"
        mpi.Wtime = lambda: __import__("time").perf_counter()
        mpi4py.MPI = mpi
        sys.modules["mpi4py"] = mpi4py
        sys.modules["mpi4py.MPI"] = mpi


def import_reference():
    """Imports and returns the reference ``pararealml`` package."""
    if not reference_available():
        raise RuntimeError(f"reference source tree not found at {REFERENCE_ROOT}")
    _install_stubs()
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    sys.dont_write_bytecode = True
    import pararealml  # noqa: F401
    import pararealml.operators.fdm  # noqa: F401
    import pararealml.operators.parareal  # noqa: F401

    return pararealml


def import_supervised_ml_operator():
    """Imports and returns the reference's ``supervised_ml_operator`` module.

    Its package ``pararealml/operators/ml/__init__.py`` imports TensorFlow
    (absent here) for the other learned operators, so the parent packages
    are registered as bare namespaces and only this module, whose own
    imports are numpy, scikit-learn and the reference itself, is loaded
    from its file."""
    import importlib

    import_reference()
    base = os.path.join(REFERENCE_ROOT, "pararealml", "operators", "ml")
    for name, path in (("pararealml.operators.ml", base),
                       ("pararealml.operators.ml.supervised", os.path.join(base, "supervised"))):
        if name not in sys.modules:
            pkg = types.ModuleType(name)
            pkg.__path__ = [path]
            sys.modules[name] = pkg
    return importlib.import_module("pararealml.operators.ml.supervised.supervised_ml_operator")


def run_ranks(size: int, fn: Callable[[], object]) -> List[object]:
    """Runs ``fn`` on ``size`` thread-ranks of the fake communicator."""
    _COMM._set(size)
    results: List[object] = [None] * size
    errors: List[BaseException] = []

    def worker(r: int):
        _COMM._local.rank = r
        try:
            results[r] = fn()
        except BaseException as e:  # pragma: no cover - surfaced below
            errors.append(e)
            if _COMM._barrier is not None:
                _COMM._barrier.abort()

    threads = [threading.Thread(target=worker, args=(r,)) for r in range(size)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    _COMM._set(1)
    if errors:
        raise errors[0]
    return results
