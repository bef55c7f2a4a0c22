"""astro_radix_sort_noalloc: the pair sort for callers that cannot allocate
device memory.

Callers whose device memory is owned by another allocator, frame loops with a
fixed preallocated budget, and embedders that forbid allocation after
start-up cannot pass the sort a temporary buffer; this entry point keeps its
scratch in a static device array of the library instead. Its results must be
exactly those of astro_radix_sort (integer keys and indices: no tolerance),
on two calls in a row, since every call reuses the array the previous call
left behind. This file is collected last and also runs on its own.
"""
from ctypes import byref, c_size_t

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_LENGTH = 1048576  # ASTRO_RADIX_SORT_NOALLOC_MAX_LENGTH


def _sorts(native, keys, idx, key_bits, count=None):
    """Both sorts of the same pairs; with `count`, the length is read on the
    device (estimated_length = len(keys)) and the first count outputs kept."""
    import torch

    from astro_gb300._native import lib, ptr

    n = len(keys)
    dk = torch.from_numpy(keys.view(np.int64)).cuda()
    di = None if idx is None else torch.from_numpy(idx.view(np.int32)).cuda()
    dc = None if count is None else torch.tensor([count], dtype=torch.int32, device="cuda")
    m = n if count is None else count
    out = []
    for noalloc in (False, True):
        ok = torch.full_like(dk, -1)
        oi = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        if noalloc:
            st = lib().astro_radix_sort_noalloc(ptr(dk), ptr(di), ptr(ok), ptr(oi), n, ptr(dc),
                                                key_bits, None)
        else:
            nbytes = c_size_t()
            assert lib().astro_radix_sort_temp_bytes(n, key_bits, byref(nbytes)) == 0
            temp = torch.empty(nbytes.value, dtype=torch.uint8, device="cuda")
            st = lib().astro_radix_sort(ptr(dk), ptr(di), ptr(ok), ptr(oi), n, ptr(dc), key_bits,
                                        ptr(temp), nbytes.value, None)
        assert st == 0
        torch.cuda.synchronize()
        k = ok.cpu().numpy().view(np.uint64)
        i = oi.cpu().numpy().view(np.uint32)
        # Slots past the device-side count are never written.
        assert (k[m:] == np.uint64(0xFFFFFFFFFFFFFFFF)).all()
        out.append((k[:m], i[:m]))
    return out


def test_noalloc_sort_equals_allocating_sort_on_consecutive_calls(native):
    rng = np.random.default_rng(2026)
    # First call: the largest accepted length, 64-bit keys with duplicates and
    # a given index array. Second call: a shorter ragged length, 18-bit keys,
    # indices 0..n-1 generated by the sort, on the scratch the first call left.
    cases = [(MAX_LENGTH, 64, True), (300_001, 18, False)]
    for n, bits, with_idx in cases:
        if bits == 64:
            keys = rng.integers(0, 1 << 63, n, dtype=np.uint64) * np.uint64(2)
        else:
            keys = rng.integers(0, 1 << bits, n, dtype=np.uint64)
        keys[rng.integers(0, n, n // 4)] = keys[1]
        idx = rng.permutation(n).astype(np.uint32) if with_idx else None
        (k_ref, i_ref), (k_na, i_na) = _sorts(native, keys, idx, bits)
        assert np.array_equal(k_na, k_ref)
        assert np.array_equal(i_na, i_ref)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(k_ref, keys[order])
        want_idx = order.astype(np.uint32) if idx is None else idx[order]
        assert np.array_equal(i_ref, want_idx)


def test_noalloc_sort_reads_the_count_on_the_device_after_a_full_call(native):
    """A count read on the device below estimated_length, right after a call
    of the maximum length left its keys and look-back words in the array."""
    rng = np.random.default_rng(7)
    full = rng.integers(0, 1 << 63, MAX_LENGTH, dtype=np.uint64)
    _sorts(native, full, None, 64)
    n, count = 300_001, 123_457
    keys = rng.integers(0, 1 << 40, n, dtype=np.uint64)
    keys[rng.integers(0, count, count // 5)] = keys[3]
    idx = rng.permutation(n).astype(np.uint32)
    (k_ref, i_ref), (k_na, i_na) = _sorts(native, keys, idx, 40, count=count)
    assert np.array_equal(k_na, k_ref) and np.array_equal(i_na, i_ref)
    order = np.argsort(keys[:count], kind="stable")
    assert np.array_equal(k_ref, keys[:count][order])
    assert np.array_equal(i_ref, idx[:count][order])


def test_noalloc_sort_reports_a_lookback_timeout(native):
    """The no-alloc sort's device status: a sort on the static array whose
    look-back waits give up (tile 0 never processed, short poll limit; the
    waits are bounded, so the GPU is never hung) is reported by
    astro_radix_sort_noalloc_status, and the next call sorts correctly."""
    import torch

    from astro_gb300._native import lib, ptr

    n = 3 * 4096 + 9
    keys = np.random.default_rng(5).integers(0, 256, n, dtype=np.uint64)
    dk = torch.from_numpy(keys.view(np.int64)).cuda()
    ok = torch.full_like(dk, -1)
    oi = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert lib().astro_test_sort_lookback_timeout(ptr(dk), ptr(ok), ptr(oi), n, 8, 4096, None, 0,
                                                  None) == 0
    assert lib().astro_radix_sort_noalloc_status(None) == -6  # ASTRO_ERR_DEVICE_TIMEOUT
    assert lib().astro_radix_sort_noalloc_status(None) == 0
    (k_ref, i_ref), (k_na, i_na) = _sorts(native, keys, None, 8)
    assert np.array_equal(k_na, k_ref) and np.array_equal(i_na, i_ref)
    assert lib().astro_radix_sort_noalloc_status(None) == 0


def test_noalloc_sort_rejects_lengths_beyond_its_maximum(native):
    import torch

    from astro_gb300._native import lib, ptr

    n = MAX_LENGTH + 1
    dk = torch.zeros(n, dtype=torch.int64, device="cuda")
    ok = torch.full_like(dk, -1)
    oi = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    assert lib().astro_radix_sort_noalloc(ptr(dk), None, ptr(ok), ptr(oi), n, None, 64, None) == -2
    torch.cuda.synchronize()
    assert (ok.cpu().numpy() == -1).all()
