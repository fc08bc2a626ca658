"""The allocation-free radix sort entry point (pp_radix_sort_noalloc),
called through the C ABI on caller-owned device buffers, must give exactly
the output of the allocating entry point (pp_radix_sort_host). It serves
callers that cannot call cudaMalloc themselves, for instance code whose
device memory belongs to a pooling allocator, or a latency-bound loop where
an allocation could synchronise the device. Two calls in a row check that
the shared scratch array is reset between calls.

This file is collected last so that a failure here comes after every other
test has run.
"""
import numpy as np
import pytest

import pphpc_gb300 as pp

pytestmark = pytest.mark.gpu

MAX_N = 1 << 22


def _noalloc_sort(torch, keys, vals, key_bits):
    dev = torch.device("cuda:0")
    k = torch.from_numpy(keys.view(np.int32).copy()).to(dev)
    v = torch.from_numpy(vals.view(np.int32).copy()).to(dev)
    ko = torch.empty_like(k)
    vo = torch.empty_like(v)
    torch.cuda.synchronize()
    rc = pp.lib().pp_radix_sort_noalloc(len(keys), k.data_ptr(), v.data_ptr(),
                                        ko.data_ptr(), vo.data_ptr(), key_bits, 0, None)
    assert rc == pp.PP_SUCCESS
    return (ko.cpu().numpy().view(np.uint32).copy(),
            vo.cpu().numpy().view(np.uint32).copy())


def test_noalloc_sort_matches_allocating_sort_twice():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2024)
    # first call: random 28-bit cell keys; second call: a different size and
    # key width, many duplicates, the maximum accepted size
    cases = [(1_000_003, 28), (MAX_N, 21)]
    for n, bits in cases:
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint32)
        if bits == 21:
            keys[::3] = 7
        vals = np.arange(n, dtype=np.uint32)
        want_k, want_v = pp.radix_sort(keys, vals, bits)
        got_k, got_v = _noalloc_sort(torch, keys, vals, bits)
        assert np.array_equal(got_k, want_k)
        assert np.array_equal(got_v, want_v)


def test_noalloc_sort_rejects_oversize():
    rc = pp.lib().pp_radix_sort_noalloc(MAX_N + 1, None, None, None, None, 28, 0, None)
    assert rc == pp.PP_INVALID_ARGS
