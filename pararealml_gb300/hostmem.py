"""Pinned host buffers on huge pages for long trajectories.

``FDMOperator.solve_into`` streams a trajectory to a caller-owned pinned
host buffer.  For buffers of tens of GB the host page size decides the
device-to-host rate on GB300 (Grace host): with the 64 KiB base pages of a
``pin_memory=True`` tensor, consecutive passes over a 31 GiB buffer ran at
193 and 105-113 GB/s in turn, while the same buffer on transparent huge
pages ran every pass at 193 GB/s (the link's rate).  ``PinnedHostBuffer``
maps anonymous memory, asks the kernel for huge pages (``MADV_HUGEPAGE``;
without transparent huge pages the call is a no-op and base pages are used),
touches every page and registers the range with CUDA.  The buffer owns the
mapping: ``close()`` (or leaving a ``with`` block) unregisters and unmaps it,
after which its tensor must not be used.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

_PROT_READ, _PROT_WRITE = 0x1, 0x2
_MAP_PRIVATE, _MAP_ANONYMOUS = 0x02, 0x20
_MADV_HUGEPAGE = 14
_HUGE = 2 << 20


def _libc():
    lib = ctypes.CDLL("libc.so.6", use_errno=True)
    lib.mmap.restype = ctypes.c_void_p
    lib.mmap.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_long]
    lib.munmap.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    lib.madvise.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    return lib


class PinnedHostBuffer:
    """A pinned host tensor of ``shape`` and ``dtype`` on huge pages.

    ``.tensor`` is a CPU torch tensor that CUDA copies treat as pinned
    (``non_blocking`` copies run asynchronously at the link's rate)."""

    def __init__(self, shape, dtype=None):
        import torch

        dtype = torch.float64 if dtype is None else dtype
        itemsize = torch.empty((), dtype=dtype).element_size()
        self.nbytes = int(math.prod(shape)) * itemsize
        self._size = max(_HUGE, (self.nbytes + _HUGE - 1) // _HUGE * _HUGE)
        self._libc = _libc()
        p = self._libc.mmap(None, self._size, _PROT_READ | _PROT_WRITE, _MAP_PRIVATE | _MAP_ANONYMOUS, -1, 0)
        if p is None or p == ctypes.c_void_p(-1).value:
            raise MemoryError(f"mmap of {self._size} bytes failed (errno {ctypes.get_errno()})")
        self._ptr = p
        self.huge_pages = self._libc.madvise(p, self._size, _MADV_HUGEPAGE) == 0
        raw = np.frombuffer((ctypes.c_char * self._size).from_address(p), dtype=np.uint8)
        raw[:: 64 << 10] = 0  # fault every page in before registering
        rc = torch.cuda.cudart().cudaHostRegister(p, self._size, 0)
        if int(rc) != 0:
            self._libc.munmap(p, self._size)
            self._ptr = None
            raise RuntimeError(f"cudaHostRegister failed ({rc})")
        self._registered = True
        self.tensor = torch.from_numpy(raw[: self.nbytes].view(_numpy_dtype(dtype))).view(tuple(shape))

    def huge_page_fraction(self) -> float:
        """Share of the mapping backed by transparent huge pages now (from
        /proc/self/smaps; 0.0 where that cannot be read)."""
        if self._ptr is None:
            return 0.0
        try:
            with open("/proc/self/smaps") as f:
                size = 0
                for line in f:
                    head = line.split(None, 1)[0]
                    if "-" in head and ":" not in head:
                        lo, hi = (int(v, 16) for v in head.split("-"))
                        size = hi - lo if lo <= self._ptr < hi else 0
                    elif size and head == "AnonHugePages:":
                        return min(1.0, int(line.split()[1]) * 1024 / size)
        except (OSError, ValueError, IndexError):
            pass
        return 0.0

    def close(self) -> None:
        """Unregisters and unmaps the buffer (its tensor is then invalid)."""
        import torch

        if self._ptr is None:
            return
        self.tensor = None
        if self._registered:
            torch.cuda.synchronize()
            torch.cuda.cudart().cudaHostUnregister(self._ptr)
            self._registered = False
        self._libc.munmap(self._ptr, self._size)
        self._ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass


def _numpy_dtype(dtype):
    import torch

    return {torch.float64: np.float64, torch.float32: np.float32, torch.int32: np.int32,
            torch.int64: np.int64, torch.uint8: np.uint8}[dtype]
