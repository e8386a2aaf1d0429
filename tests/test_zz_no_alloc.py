"""The allocation-free perfect-hash entry point (cgs_perfect_hash_build_noalloc).

Callers that cannot allocate device memory when they need a table (code in an
allocator callback, where allocating would re-enter the allocator, or a
service that reserves its device memory at start-up) use this entry point:
its working memory is a fixed array inside the library.  The tests call it
through the C ABI and check, on two calls in a row with different sizes, that
its tables, parameters and status codes are those of the allocating entry
point cgs_perfect_hash_build: on consecutive keys, on BVH key sets that need
many trials, and on key sets where the build fails.  Inputs above the fixed
capacity are refused.  The file is collected last, and passes both alone in a
fresh process and after the other tests.
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


def _bvh_keys(leaves):
    from cgspline_gb300 import scenes
    return scenes.bvh_keys(leaves)


def test_noalloc_matches_on_keys_that_need_many_trials(lib, torch):
    # BVH heap-key sets of 20,000 and 3,000 leaves: the build succeeds only at
    # its 15th and 11th trial, so every trial's reset of the shared scratch
    # is exercised; two calls in a row.
    for leaves in (20000, 3000):
        keys = _bvh_keys(leaves)
        ref = build(lib, "cgs_perfect_hash_build", keys, torch)
        got = build(lib, "cgs_perfect_hash_build_noalloc", keys, torch)
        assert ref[0] == 0 and got[0] == 0
        assert got[1][4] > 0
        assert np.array_equal(ref[1], got[1])
        assert np.array_equal(ref[2], got[2])
        assert np.array_equal(ref[3], got[3])


def test_noalloc_failures_match_allocating_build(lib, torch):
    # 533 leaves: no injective table in 16 trials (CGS_ERR_HASH_FAILED).
    # Seeded random keys: more than 4 keys share a bucket
    # (CGS_ERR_HASH_BUCKET_OVERFLOW).  Then a good key set on the same
    # scratch still matches.
    rng = np.random.default_rng(7)
    rand = np.unique(rng.integers(1, 2 ** 32 - 1, size=200000, dtype=np.uint64)).astype(np.uint32)
    for keys, status in ((_bvh_keys(533), 6), (rand, 5), (_bvh_keys(1000), 0)):
        ref = build(lib, "cgs_perfect_hash_build", keys, torch)
        got = build(lib, "cgs_perfect_hash_build_noalloc", keys, torch)
        assert ref[0] == status and got[0] == status
        assert np.array_equal(ref[1], got[1])
        if status == 0:
            assert np.array_equal(ref[2], got[2]) and np.array_equal(ref[3], got[3])


def test_noalloc_rejects_inputs_above_capacity(lib, torch):
    keys = torch.arange(1, MAX_KEYS + 2, dtype=torch.int32, device="cuda")
    disp = torch.zeros(MAX_KEYS, dtype=torch.int32, device="cuda")
    table = torch.zeros(2 * MAX_KEYS, dtype=torch.int32, device="cuda")
    par = np.zeros(5, np.uint32)
    st = lib.cgs_perfect_hash_build_noalloc(C.c_void_p(keys.data_ptr()), MAX_KEYS + 1, C.c_void_p(disp.data_ptr()),
                                            MAX_KEYS, C.c_void_p(table.data_ptr()), 2 * MAX_KEYS,
                                            par.ctypes.data_as(C.c_void_p), None)
    assert st == 12  # CGS_ERR_CAPACITY
