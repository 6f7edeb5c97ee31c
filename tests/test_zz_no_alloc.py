"""gs_radix_sort_no_alloc: the sort for callers that cannot call cudaMalloc (its scratch is a
static device array inside the library, at most 2^20 pairs).  Called through the C ABI and
checked bit for bit against gs_radix_sort with caller-provided scratch, on calls in a row of
growing and shrinking sizes and key widths (the array keeps the previous call's contents, which
the entry point must not depend on).  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1 << 20


def _keys(n, seed):
    rng = np.random.default_rng(seed)
    keys = rng.random(n).astype(np.float32).view(np.uint32).copy()
    keys[rng.integers(0, n, size=n // 4)] = keys[0]  # ties
    vals = rng.permutation(n).astype(np.uint32)
    return keys, vals


def _dev(torch, a):
    return torch.from_numpy(a.view(np.int32).copy()).cuda()


def _with_caller_scratch(gs, torch, keys, vals, count=None, key_bits=32):
    dk, dv = _dev(torch, keys), _dev(torch, vals)
    nb = gs.RadixSorter.scratch_bytes(len(keys))
    scratch = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    gs.RadixSorter.sort(dk, dv, len(keys), scratch, nb, count=count, key_bits=key_bits)
    torch.cuda.synchronize()
    return dk.cpu().numpy().view(np.uint32), dv.cpu().numpy().view(np.uint32)


def _no_alloc(gs, torch, keys, vals, count=None, key_bits=32):
    dk, dv = _dev(torch, keys), _dev(torch, vals)
    cnt = None if count is None else ctypes.c_void_p(int(count.data_ptr()))
    st = gs.lib().gs_radix_sort_no_alloc(ctypes.c_void_p(dk.data_ptr()), ctypes.c_void_p(dv.data_ptr()), len(keys), cnt,
                                         key_bits, None)
    assert st == 0, gs.lib().gs_last_error()
    torch.cuda.synchronize()
    return dk.cpu().numpy().view(np.uint32), dv.cpu().numpy().view(np.uint32)


def test_no_alloc_sort_matches_caller_scratch_sort_twice(gs, cuda):
    torch = cuda
    for seed, n in ((1, 300_001), (2, LIMIT)):  # two calls in a row, different sizes and data
        keys, vals = _keys(n, seed)
        a = _with_caller_scratch(gs, torch, keys, vals)
        b = _no_alloc(gs, torch, keys, vals)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(b[0], keys[order]) and np.array_equal(b[1], vals[order])


def test_no_alloc_sort_sizes_and_key_bits_in_any_order(gs, cuda):
    """Calls that shrink and grow the sort's layout inside the one static array, with values that
    make the pairs left behind read as look-back flags of any of the first 1024 epochs."""
    torch = cuda
    for n, bits, seed in ((LIMIT, 32, 11), (100_000, 32, 12), (LIMIT, 32, 13), (50_000, 12, 14), (LIMIT, 20, 15),
                          (3_840, 7, 16), (LIMIT, 32, 17)):
        rng = np.random.default_rng(seed)
        keys = rng.integers(0, 1 << bits, size=n, dtype=np.uint64).astype(np.uint32)
        keys[rng.integers(0, n, size=n // 4)] = keys[0]
        vals = (4 * (1 + (np.arange(n, dtype=np.uint32) % 1024)) + 1).astype(np.uint32)
        a = _with_caller_scratch(gs, torch, keys, vals, key_bits=bits)
        b = _no_alloc(gs, torch, keys, vals, key_bits=bits)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(b[0], keys[order]) and np.array_equal(b[1], vals[order])


def test_no_alloc_sort_device_count(gs, cuda):
    torch = cuda
    keys, vals = _keys(50_000, 3)
    count = torch.tensor([12_345], dtype=torch.int32, device="cuda")
    a = _with_caller_scratch(gs, torch, keys, vals, count=count)
    b = _no_alloc(gs, torch, keys, vals, count=count)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_no_alloc_sort_rejects_sizes_beyond_its_limit(gs, cuda):
    st = gs.lib().gs_radix_sort_no_alloc(None, None, LIMIT + 1, None, 32, None)
    assert st == 1 and b"1048576" in gs.lib().gs_last_error()
