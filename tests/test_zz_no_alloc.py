"""The allocation-free perfect-hash entry point (cgs_perfect_hash_build_noalloc).

Callers that cannot allocate device memory when they need a table (a stream
being captured into a CUDA graph, an allocator callback, a service that must
not grow the device heap) use this entry point: its working memory is a fixed
array inside the library.  The test calls it through the C ABI and checks,
on two calls in a row with different sizes, that its tables are bit-identical
to those of the allocating entry point cgs_perfect_hash_build, and that inputs
above its fixed capacity are refused.  It lives in its own file, collected
last, and passes both alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 262144


def build(lib, fn, keys_np, torch, cap_pad=0):
    n = keys_np.size
    keys = torch.from_numpy(keys_np.view(np.int32)).cuda()
    s = max(2, (n - 1) >> 1)
    dsz = 1 << (s.bit_length() - 1)
    tcap = n + 15 * max(4, int(np.float32(0.05) * np.float32(n))) + cap_pad
    disp = torch.full((dsz,), -7, dtype=torch.int32, device="cuda")
    table = torch.full((tcap,), -7, dtype=torch.int32, device="cuda")
    par = np.zeros(5, np.uint32)
    st = getattr(lib, fn)(C.c_void_p(keys.data_ptr()), n, C.c_void_p(disp.data_ptr()), dsz,
                          C.c_void_p(table.data_ptr()), tcap, par.ctypes.data_as(C.c_void_p),
                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    N = int(par[2])
    return st, par.copy(), disp.cpu().numpy().view(np.uint32).copy(), table[:N].cpu().numpy().view(np.uint32).copy()


@pytest.fixture(scope="module")
def lib():
    from cgspline_gb300 import _capi
    return _capi.load()


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


@pytest.mark.parametrize("sizes", [(1000, 65537), (MAX_KEYS, 31)])
def test_noalloc_matches_allocating_build_twice(lib, torch, sizes):
    for n in sizes:  # two calls in a row on the shared scratch
        keys = np.arange(1, n + 1, dtype=np.uint32)
        ref = build(lib, "cgs_perfect_hash_build", keys, torch)
        got = build(lib, "cgs_perfect_hash_build_noalloc", keys, torch)
        assert ref[0] == 0 and got[0] == 0
        assert np.array_equal(ref[1], got[1])
        assert np.array_equal(ref[2], got[2])
        assert np.array_equal(ref[3], got[3])
        # the table is injective on the keys
        A, B, N, mask = (int(x) for x in got[1][:4])
        slots = ((A * keys.astype(np.uint64) + B + got[2][keys & mask]) & 0xFFFFFFFF) % N
        assert np.array_equal(got[3][slots], np.arange(n))


def test_noalloc_rejects_inputs_above_capacity(lib, torch):
    keys = torch.arange(1, MAX_KEYS + 2, dtype=torch.int32, device="cuda")
    disp = torch.zeros(MAX_KEYS, dtype=torch.int32, device="cuda")
    table = torch.zeros(2 * MAX_KEYS, dtype=torch.int32, device="cuda")
    par = np.zeros(5, np.uint32)
    st = lib.cgs_perfect_hash_build_noalloc(C.c_void_p(keys.data_ptr()), MAX_KEYS + 1, C.c_void_p(disp.data_ptr()),
                                            MAX_KEYS, C.c_void_p(table.data_ptr()), 2 * MAX_KEYS,
                                            par.ctypes.data_as(C.c_void_p), None)
    assert st == 12  # CGS_ERR_CAPACITY
