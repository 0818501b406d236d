"""pg_reduce_sum_noalloc through the C ABI.

The entry point exists for callers that cannot allocate device memory (their
device memory belongs to another allocator, or they cannot take cudaMalloc's
implicit synchronisation): it sums a device array into a device scalar using
only a fixed scratch array inside the library.  The test owns the input and
output buffers (allocated here with torch); the entry point allocates nothing.
Two calls in a row must agree with pg_reduce_sum on the same data, whose
summation order is the same, so the comparison is exact; after a warm-up call
(the first call may load the module), a call leaves the device's free memory
unchanged.  n = 0 writes exactly 0.0.  This file is
collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 1 << 28


def _entry(lib):
    fn = lib.pg_reduce_sum_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def test_noalloc_sum_matches_reduce_sum_on_two_calls(lib, ctx):
    torch = pytest.importorskip("torch")
    fn = _entry(lib)
    rng = np.random.default_rng(2027)
    stream = torch.cuda.current_stream()
    for n in (3 * 2048 + 5, (1 << 20) + 77):
        x = rng.standard_normal(n) * 10.0 ** rng.uniform(-4, 4, n)
        expect = ctx.reduce_sum(x)
        dx = torch.from_numpy(x).to("cuda")
        dout = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        assert fn(dx.data_ptr(), n, dout.data_ptr(), stream.cuda_stream) == 0
        torch.cuda.synchronize()
        got = float(dout.cpu().numpy()[0])
        assert got == expect, (n, got, expect)


def test_noalloc_sum_allocates_nothing(lib):
    torch = pytest.importorskip("torch")
    fn = _entry(lib)
    x = torch.arange(1 << 20, dtype=torch.float64, device="cuda")
    dout = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert fn(x.data_ptr(), x.numel(), dout.data_ptr(), None) == 0  # warm-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    assert fn(x.data_ptr(), x.numel(), dout.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert float(dout.cpu()[0]) == float(x.numel() * (x.numel() - 1) // 2)


def test_noalloc_sum_of_nothing_is_zero(lib):
    torch = pytest.importorskip("torch")
    fn = _entry(lib)
    dx = torch.zeros(1, dtype=torch.float64, device="cuda")
    dout = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
    assert fn(dx.data_ptr(), 0, dout.data_ptr(), None) == 0
    torch.cuda.synchronize()
    got = float(dout.cpu()[0])
    assert got == 0.0 and not np.signbit(got)


def test_noalloc_sum_rejects_sizes_above_the_limit(lib):
    torch = pytest.importorskip("torch")
    fn = _entry(lib)
    dout = torch.zeros(1, dtype=torch.float64, device="cuda")
    dx = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert fn(dx.data_ptr(), MAX_N + 1, dout.data_ptr(), None) == -1  # PG_BAD_ARG, nothing launched
