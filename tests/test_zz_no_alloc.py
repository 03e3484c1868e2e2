"""The allocation-free Parareal norm, through the C ABI (needs a GB300).

``prml_pr_update_norm_noalloc`` serves callers that cannot allocate device
memory where they need the Parareal update norm (a host binding that owns
every device buffer, or a run that forbids new allocations): it keeps its
partial sums in a fixed array inside the library.  This test checks it
against the allocating entry point on two calls in a row with different
shapes, so a second call cannot lean on what the first one left in the
shared array, and checks that oversized requests are refused.  It lives in
its own file, collected last, and passes alone or after the other tests.
"""

import ctypes

import pytest

from pararealml_gb300 import _native

pytestmark = pytest.mark.gpu


def test_noalloc_norm_matches_the_allocating_norm_on_two_calls():
    import torch

    _native.build()
    lib = _native.lib()
    stream = torch.cuda.current_stream().cuda_stream
    gen = torch.Generator(device="cuda").manual_seed(7)
    for S, B, C, nx, ny, pitch, chunks in ((4, 3, 2, 37, 45, 64, 3), (2, 5, 1, 129, 70, 96, 5)):
        new = torch.randn((S, B, C, nx, pitch), dtype=torch.float64, device="cuda", generator=gen)
        old = torch.randn((S, B, C, nx, pitch), dtype=torch.float64, device="cuda", generator=gen)
        partial = torch.empty(lib.prml_pr_norm_scratch_elems(S, B, C, chunks), dtype=torch.float64, device="cuda")
        want = torch.empty((B, C), dtype=torch.float64, device="cuda")
        got = torch.full((B, C), float("nan"), dtype=torch.float64, device="cuda")
        _native.check(
            lib.prml_pr_update_norm(new.data_ptr(), old.data_ptr(), S, B, C, nx, ny, pitch, chunks,
                                    partial.data_ptr(), want.data_ptr(), stream),
            "norm",
        )
        _native.check(
            lib.prml_pr_update_norm_noalloc(new.data_ptr(), old.data_ptr(), S, B, C, nx, ny, pitch,
                                            chunks, got.data_ptr(), stream),
            "norm (no alloc)",
        )
        torch.cuda.synchronize()
        assert torch.allclose(got, want, rtol=1e-12, atol=0.0)
        assert bool(torch.all(got > 0))


def test_noalloc_norm_refuses_requests_beyond_its_scratch():
    import torch

    _native.build()
    lib = _native.lib()
    x = torch.zeros((1, 1, 1, 4, 32), dtype=torch.float64, device="cuda")
    out = torch.zeros((1, 1), dtype=torch.float64, device="cuda")
    too_many_chunks = 262144 + 1
    rc = lib.prml_pr_update_norm_noalloc(x.data_ptr(), x.data_ptr(), 1, 1, 1, 4, 4, 32, too_many_chunks,
                                         out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == _native.PRML_ERR_ARG
    assert b"exceeds its fixed scratch" in lib.prml_last_error()
