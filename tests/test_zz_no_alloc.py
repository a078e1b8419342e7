"""The allocation-free selection entry point (bgt_gpu_select_noalloc).

It serves callers that cannot allocate device memory -- code inside a stream
capture, processes whose device memory belongs to another allocator, loops
that must not take the driver's allocation locks -- by working in a fixed
static scratch array of the library.  This test calls it through the C ABI
on caller-owned device buffers and checks, on two calls in a row (the second
on a different lattice size, so stale scratch from the first would show),
that it selects what the regular entry point (bgt_gpu_lattice_select on a
lattice built from the same prior) selects.  Collected last on purpose: if it
fails, a run stopping at the first failure has run everything else.
"""
import ctypes

import numpy as np
import pytest

import bayesiangrouptesting_gb300 as bgt

pytestmark = pytest.mark.gpu


def _regular_selection(n, pi0):
    lat = bgt.Lattice(bgt.LatticeType.replicated_non_dilution, n, pi0)
    return lat, bgt.reverse_bits(lat.select_experiment(bgt.SelectorType.op_bha), n)


def test_select_noalloc_matches_regular_entry_point(gpu):
    torch = pytest.importorskip("torch")
    lib = gpu
    rng = np.random.default_rng(4242)
    out = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    for call, n in enumerate((16, 18)):
        pi0 = rng.uniform(0.01, 0.2, n)
        lat, want = _regular_selection(n, pi0)
        # The fresh lattice holds the raw prior (no normalisation), so its
        # posterior read back is exactly what the regular path selected on.
        post = torch.from_numpy(lat.posterior()).to("cuda")
        status = lib.bgt_gpu_select_noalloc(ctypes.c_void_p(post.data_ptr()), n, 1, ctypes.c_void_p(out.data_ptr()),
                                            ctypes.c_void_p(stream.cuda_stream))
        assert status == 0, lib.bgt_gpu_last_error()
        torch.cuda.synchronize()
        got = int(out.item()) & 0xFFFFFFFF
        assert got == want, (call, n, got, want)


def test_select_noalloc_rejects_oversized_lattices(gpu):
    torch = pytest.importorskip("torch")
    lib = gpu
    post = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.int32, device="cuda")
    status = lib.bgt_gpu_select_noalloc(ctypes.c_void_p(post.data_ptr()), 21, 1, ctypes.c_void_p(out.data_ptr()), None)
    assert status == 2
    assert b"20" in lib.bgt_gpu_last_error()
