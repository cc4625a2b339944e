"""The allocation-free bitset count, called through the C ABI, against the allocating one.

sg_bitset_count_noalloc serves callers that must not allocate device memory (a process whose device
memory belongs to another allocator with a fixed budget, or a latency-critical path that cannot take
the device-wide synchronisation of cudaMalloc / cudaFree): it keeps its per-block partial sums in a
fixed array inside the library instead of allocating them.  Two calls in a row must give the same counts as
sg_bitset_count (integer work: exact), the second with fewer chunks than the first so that stale
partial sums left in the shared array by the first call would show; sizes beyond the array's limit
are refused.  This file is collected last and passes alone in a fresh process as well.
"""

import ctypes

import pytest
import torch

import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N

pytestmark = pytest.mark.gpu

MAX_BITS = 1 << 34  # 8192 partial sums x 65536 blocks x 32 bits


def _count_allocating(lib, words: torch.Tensor, nbits: int, stream) -> int:
    out = ctypes.c_int64()
    N.check(lib.sg_bitset_count(ctypes.c_void_p(words.data_ptr()), nbits, stream, ctypes.byref(out)),
            "sg_bitset_count")
    return out.value


def test_noalloc_count_matches_allocating_count_twice():
    lib = sg.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    gen = torch.Generator(device="cuda").manual_seed(11)
    # first call: 2^31 + 77 bits (many chunks, a partial tail word); second: fewer chunks, odd size
    for nbits in [(1 << 31) + 77, (1 << 24) + 12345]:
        nwords = (nbits + 31) // 32
        words = torch.randint(-(2**31), 2**31, (nwords,), dtype=torch.int32, device="cuda", generator=gen)
        out = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        live = sg.live_device_allocations()
        st = lib.sg_bitset_count_noalloc(ctypes.c_void_p(words.data_ptr()), nbits,
                                         ctypes.c_void_p(out.data_ptr()), stream)
        assert st == N.SG_OK
        torch.cuda.synchronize()
        assert sg.live_device_allocations() == live  # nothing taken from the library's allocator
        assert int(out.item()) == _count_allocating(lib, words, nbits, stream)


def test_noalloc_count_refuses_beyond_limit_and_handles_empty():
    lib = sg.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    words = torch.zeros(4, dtype=torch.int32, device="cuda")
    out = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    st = lib.sg_bitset_count_noalloc(ctypes.c_void_p(words.data_ptr()), MAX_BITS + 1,
                                     ctypes.c_void_p(out.data_ptr()), stream)
    assert st == N.SG_ERR_BAD_ARG
    st = lib.sg_bitset_count_noalloc(ctypes.c_void_p(words.data_ptr()), 0, ctypes.c_void_p(out.data_ptr()), stream)
    assert st == N.SG_OK
    torch.cuda.synchronize()
    assert int(out.item()) == 0
