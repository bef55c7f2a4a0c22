"""Device status of the stand-alone sort.

Every decoupled look-back wait of the sort is bounded. The test hook
astro_test_sort_lookback_timeout queues a one-pass sort whose tile 0 is never
processed, so the later tiles' look-backs wait on a status word that nothing
publishes and give up after a short poll limit: the GPU is neither faulted
nor hung, and the sort must report ASTRO_ERR_DEVICE_TIMEOUT through
astro_radix_sort_status. The same temporaries then sort correctly again.
"""
from ctypes import byref, c_size_t

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_DEVICE_TIMEOUT = -6
SPIN_LIMIT = 4096  # polls before a look-back wait gives up (about a millisecond)


def _buffers(n, key_bits, seed):
    import torch

    rng = np.random.default_rng(seed)
    keys = rng.integers(0, 1 << key_bits, n, dtype=np.uint64)
    dk = torch.from_numpy(keys.view(np.int64)).cuda()
    ok = torch.full_like(dk, -1)
    oi = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    return keys, dk, ok, oi


def test_lookback_timeout_is_reported_and_the_scratch_stays_usable(native):
    import torch

    from astro_gb300._native import lib, ptr

    n, bits = 3 * 4096 + 17, 8  # several tiles, one pass
    keys, dk, ok, oi = _buffers(n, bits, 11)
    nbytes = c_size_t()
    assert lib().astro_radix_sort_temp_bytes(n, bits, byref(nbytes)) == 0
    temp = torch.empty(nbytes.value, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    torch.cuda.synchronize()  # the buffers' fills (default stream) come first
    assert lib().astro_test_sort_lookback_timeout(ptr(dk), ptr(ok), ptr(oi), n, bits, SPIN_LIMIT,
                                                  ptr(temp), nbytes.value, sp) == 0
    assert lib().astro_radix_sort_status(ptr(temp), sp) == ERR_DEVICE_TIMEOUT
    # Read and cleared: the next query is clean.
    assert lib().astro_radix_sort_status(ptr(temp), sp) == 0
    # Every store of the stalled sort stayed inside the output: the slots it
    # wrote hold input keys.
    got = ok.cpu().numpy().view(np.uint64)
    written = got != np.uint64(0xFFFFFFFFFFFFFFFF)
    assert np.isin(got[written], keys).all()
    idx = oi.cpu().numpy()
    assert ((idx[written] >= 0) & (idx[written] < n)).all()
    # The same scratch sorts correctly afterwards, on a side stream and on
    # the NULL stream (which reports the status from the call itself).
    want = np.argsort(keys, kind="stable")
    for s in (sp, None):
        ok.fill_(-1)
        oi.fill_(-1)
        torch.cuda.synchronize()
        assert lib().astro_radix_sort(ptr(dk), None, ptr(ok), ptr(oi), n, None, bits, ptr(temp),
                                      nbytes.value, s) == 0
        assert lib().astro_radix_sort_status(ptr(temp), s) == 0
        torch.cuda.synchronize()
        assert np.array_equal(ok.cpu().numpy().view(np.uint64), keys[want])
        assert np.array_equal(oi.cpu().numpy().view(np.uint32), want.astype(np.uint32))


def test_radix_sort_status_through_the_python_sorter(native):
    import torch

    from astro_gb300 import AstroError
    from astro_gb300._native import lib, ptr
    from astro_gb300.radix_sort import RadixSort

    n, bits = 2 * 4096 + 5, 8
    keys, dk, ok, oi = _buffers(n, bits, 12)
    s = RadixSort(n, bits)
    s.sort(dk, None, ok, oi, n)  # NULL stream: checked by the call
    s.status()
    assert lib().astro_test_sort_lookback_timeout(ptr(dk), ptr(ok), ptr(oi), n, bits, SPIN_LIMIT,
                                                  ptr(s.temp), s.temp.numel(), None) == 0
    with pytest.raises(AstroError) as e:
        s.status()
    assert e.value.status == ERR_DEVICE_TIMEOUT
    torch.cuda.synchronize()
