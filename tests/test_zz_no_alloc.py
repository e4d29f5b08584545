"""The allocation-free radix sort entry point against the allocating one, through the C ABI.

pcisph_radixsort_enqueue_noalloc exists for callers that must not allocate device memory while they sort
(a pool allocator owns the device's memory, or an allocation would stall a latency-critical loop); its
scratch is a fixed array inside the library. This file is collected last so that a run stopping at the
first failure has run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from pcisph_gb300 import RadixSort, _lib

pytestmark = pytest.mark.gpu
MAX = 1 << 20  # PCISPH_NOALLOC_SORT_MAX_ELEMENTS


def _dev(a):
    torch = pytest.importorskip("torch")
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _noalloc(keys, vals, n, max_bits):
    L = _lib.load()
    return L.pcisph_radixsort_enqueue_noalloc(C.c_void_p(keys.data_ptr()), C.c_void_p(vals.data_ptr()), n,
                                              max_bits, None)


def test_noalloc_sort_matches_allocating_sort_twice():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2024)
    ref_sorter = None
    # two calls in a row with different inputs: the second must not see anything left by the first. The
    # first no-alloc call comes before the allocating sorter exists, so in a fresh process it is the call
    # that finds the library's scratch with nothing else of the library set up on the device.
    for n, hi, bits in [(MAX, 1 << 19, 19), (300001, 1 << 32, 0)]:
        keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
        vals = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
        k1, v1 = _dev(keys.view(np.int32)), _dev(vals.view(np.int32))
        k2, v2 = k1.clone(), v1.clone()
        assert _noalloc(k1, v1, n, bits) == _lib.OK, _lib.load().pcisph_last_error()
        torch.cuda.synchronize()
        if ref_sorter is None:
            ref_sorter = RadixSort(0)
        ref_sorter.enqueue(k2, v2, n, max_bits=bits)
        torch.cuda.synchronize()
        # integer results: exact agreement (tolerance zero)
        np.testing.assert_array_equal(k1.cpu().numpy(), k2.cpu().numpy())
        np.testing.assert_array_equal(v1.cpu().numpy(), v2.cpu().numpy())
        order = np.argsort(keys, kind="stable")
        np.testing.assert_array_equal(k1.cpu().numpy().view(np.uint32), keys[order])


def test_noalloc_sort_rejects_more_than_its_maximum():
    torch = pytest.importorskip("torch")
    k = torch.zeros(MAX + 1, dtype=torch.int32, device="cuda")
    v = torch.zeros(MAX + 1, dtype=torch.int32, device="cuda")
    assert _noalloc(k, v, MAX + 1, 0) == _lib.ERR_INVALID_ARG
    assert b"exceed its fixed scratch" in _lib.load().pcisph_last_error()


def test_noalloc_sort_argument_checks():
    """Bad arguments come back as status codes before any work is queued; an empty sort is a no-op."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    k = torch.arange(64, 0, -1, dtype=torch.int32, device="cuda")
    v = torch.arange(64, dtype=torch.int32, device="cuda")
    assert _noalloc(k, v, 64, 33) == _lib.ERR_INVALID_ARG
    assert b"max_bits" in L.pcisph_last_error()
    assert L.pcisph_radixsort_enqueue_noalloc(None, C.c_void_p(v.data_ptr()), 64, 0, None) == _lib.ERR_INVALID_ARG
    assert L.pcisph_radixsort_enqueue_noalloc(C.c_void_p(k.data_ptr()), None, 64, 0, None) == _lib.ERR_INVALID_ARG
    assert L.pcisph_radixsort_enqueue_noalloc(None, None, 0, 0, None) == _lib.OK
    assert _noalloc(k, v, 0, 0) == _lib.OK
    torch.cuda.synchronize()
    # nothing was touched by the rejected or empty calls
    np.testing.assert_array_equal(k.cpu().numpy(), np.arange(64, 0, -1))
    np.testing.assert_array_equal(v.cpu().numpy(), np.arange(64))
    # and the same array then sorts
    assert _noalloc(k, v, 64, 7) == _lib.OK
    torch.cuda.synchronize()
    np.testing.assert_array_equal(k.cpu().numpy(), np.arange(1, 65))
    np.testing.assert_array_equal(v.cpu().numpy(), np.arange(63, -1, -1))
