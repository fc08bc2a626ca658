"""The allocation-free radix sort entry point (pp_radix_sort_noalloc),
called through the C ABI on caller-owned device buffers, must give exactly
the output of the allocating entry point (pp_radix_sort_host) and of a
stable argsort on the host. It serves callers that cannot call cudaMalloc
themselves, for instance code whose device memory belongs to a pooling
allocator, or a latency-bound loop where an allocation could synchronise the
device. Calls come in a row, so the shared scratch array must be reset
between them.

This file is collected last so that a failure here comes after every other
test has run.
"""
import numpy as np
import pytest

import pphpc_gb300 as pp

MAX_N = 1 << 22
SORT_TILE = 4096          # elements one sort CTA handles


def _noalloc_sort(torch, keys, vals, key_bits, digit_bits=0):
    dev = torch.device("cuda:0")
    n = len(keys)
    k = torch.from_numpy(keys.view(np.int32).copy()).to(dev)
    v = torch.from_numpy(vals.view(np.int32).copy()).to(dev)
    ko = torch.empty_like(k)
    vo = torch.empty_like(v)
    torch.cuda.synchronize()
    ptr = (lambda t: t.data_ptr()) if n else (lambda t: None)
    rc = pp.lib().pp_radix_sort_noalloc(n, ptr(k), ptr(v), ptr(ko), ptr(vo),
                                        key_bits, digit_bits, None)
    assert rc == pp.PP_SUCCESS
    return (ko.cpu().numpy().view(np.uint32).copy(),
            vo.cpu().numpy().view(np.uint32).copy())


def _stable(keys, vals, key_bits):
    mask = np.uint64((1 << key_bits) - 1)
    order = np.argsort(keys.astype(np.uint64) & mask, kind="stable")
    return keys[order], vals[order]


@pytest.mark.gpu
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
        sk, sv = _stable(keys, vals, bits)
        assert np.array_equal(got_k, sk) and np.array_equal(got_v, sv)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [0, 1, SORT_TILE - 1, SORT_TILE, SORT_TILE + 1,
                               3 * SORT_TILE + 17])
def test_noalloc_sort_edge_sizes(n):
    """Empty, single and tile-edge sizes, each sorted twice in a row."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n + 5)
    for bits in (13, 28):
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint32)
        vals = rng.integers(0, 1 << 32, n, dtype=np.uint32)
        got_k, got_v = _noalloc_sort(torch, keys, vals, bits)
        sk, sv = _stable(keys, vals, bits)
        assert np.array_equal(got_k, sk) and np.array_equal(got_v, sv), (n, bits)


@pytest.mark.gpu
@pytest.mark.parametrize("digit_bits", [5, 6, 7, 8])
def test_noalloc_sort_digit_widths_and_32_bit_keys(digit_bits):
    """Full 32-bit keys (odd and even pass counts), and 19-bit keys whose
    last digit is narrower than the digit width."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(digit_bits)
    n = 50_000
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    keys[::5] = 0xffffffff
    keys[1::7] = 0
    vals = np.arange(n, dtype=np.uint32)
    got_k, got_v = _noalloc_sort(torch, keys, vals, 32, digit_bits)
    sk, sv = _stable(keys, vals, 32)
    assert np.array_equal(got_k, sk) and np.array_equal(got_v, sv)
    keys &= np.uint32((1 << 19) - 1)
    got_k, got_v = _noalloc_sort(torch, keys, vals, 19, digit_bits)
    sk, sv = _stable(keys, vals, 19)
    assert np.array_equal(got_v, sv) and np.array_equal(got_k, sk)


def test_noalloc_sort_rejects_bad_arguments():
    # checked before any device work, so this needs no GPU
    L = pp.lib()
    assert L.pp_radix_sort_noalloc(MAX_N + 1, None, None, None, None, 28, 0, None) \
        == pp.PP_INVALID_ARGS
    assert L.pp_radix_sort_noalloc(10, None, None, None, None, 28, 0, None) \
        == pp.PP_INVALID_ARGS
    assert L.pp_radix_sort_noalloc(0, None, None, None, None, 0, 0, None) \
        == pp.PP_INVALID_ARGS
    assert L.pp_radix_sort_noalloc(0, None, None, None, None, 33, 0, None) \
        == pp.PP_INVALID_ARGS
    assert L.pp_radix_sort_noalloc(0, None, None, None, None, 28, 9, None) \
        == pp.PP_INVALID_ARGS
    assert L.pp_radix_sort_noalloc(0, None, None, None, None, 28, 4, None) \
        == pp.PP_INVALID_ARGS
    assert L.pp_radix_sort_noalloc(0, None, None, None, None, 28, 0, None) \
        == pp.PP_SUCCESS
