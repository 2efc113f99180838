"""pgs_large_hits_static (no allocation) against pgs_large_hits and the
oracle's modulo_search_euclid_all_large, through the C ABI.

Collected last on purpose (file name): it must give the same results when it
runs alone and after every other test has used the device.
"""
from __future__ import annotations

import ctypes

import pytest

import pgo
import pgsieve

pytestmark = pytest.mark.gpu

STATIC_MAX = 1 << 16


@pytest.fixture(scope="module")
def ctx():
    lib = pgsieve.load()
    h = ctypes.c_void_p()
    assert lib.pgs_create(0, ctypes.byref(h)) == pgsieve.PGS_OK
    yield lib, h
    lib.pgs_destroy(h)


def _call(lib, h, fn, M, max_mi, SL, prime, r, cap):
    mi = (ctypes.c_uint32 * max(1, cap))()
    md = (ctypes.c_uint64 * max(1, cap))()
    n = ctypes.c_size_t(123456789)
    rc = getattr(lib, fn)(h, M, max_mi, SL, prime, r, mi, md, cap, ctypes.byref(n))
    k = min(n.value, cap)
    return rc, n.value, list(zip(mi[:k], md[:k]))


CASES = [
    # (M, max_mi, SL, prime, base_r): 49,979 hits; 175 hits; 34-bit prime,
    # 464 hits; 45-bit prime, 9 hits; a prime just above 4*SL+2 over 3e8
    # values of m (about 1.5e8 hits, the first 65,536 returned)
    (1234567, 100000, 5000, 20011, 7919),
    (98765431, 10_000_000, 20000, 2_000_000_011, 1_234_567_891),
    (5, 4_000_000_000, 1000, 17_179_869_209, 9_876_543_210),
    (77, 4_000_000_000, 40000, 35_184_372_088_891, 12_345_678_901_234),
    (3, 300_000_000, 5000, 20011, 12345),
]


@pytest.fixture(scope="module")
def oracle_hits():
    """The oracle's count and first hits per case (computed once)."""
    out = {}
    for case in CASES:
        n = pgo.all_large_count(*case)
        out[case] = (n, pgo.all_large(*case, cap=STATIC_MAX))
    return out


@pytest.mark.parametrize("case", CASES)
def test_static_matches_allocating_entry_and_oracle_twice(ctx, oracle_hits, case):
    lib, h = ctx
    n, hits = oracle_hits[case]
    want = _call(lib, h, "pgs_large_hits", *case, STATIC_MAX)
    assert want == (pgsieve.PGS_OK, n, [tuple(x) for x in hits])
    first = _call(lib, h, "pgs_large_hits_static", *case, STATIC_MAX)
    second = _call(lib, h, "pgs_large_hits_static", *case, STATIC_MAX)
    assert first == want
    assert second == want


def test_static_leaves_device_memory_unchanged(ctx):
    """Free device memory is the same before and after a run of calls (after
    one warm-up call has loaded the kernels)."""
    torch = pytest.importorskip("torch")
    lib, h = ctx
    for case in CASES[:2]:
        assert _call(lib, h, "pgs_large_hits_static", *case, STATIC_MAX)[0] == pgsieve.PGS_OK
    torch.cuda.synchronize(0)
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(5):
        for case in CASES[:4]:
            assert _call(lib, h, "pgs_large_hits_static", *case, STATIC_MAX)[0] == pgsieve.PGS_OK
    torch.cuda.synchronize(0)
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0


def test_static_back_to_back_different_jobs(ctx):
    """A call after a larger one must not see the earlier hits or count."""
    lib, h = ctx
    big, small = CASES[0], CASES[1]
    assert _call(lib, h, "pgs_large_hits_static", *big, STATIC_MAX)[1] > 1000
    got = _call(lib, h, "pgs_large_hits_static", *small, STATIC_MAX)
    assert got == _call(lib, h, "pgs_large_hits", *small, STATIC_MAX)


def test_static_truncates_like_allocating_entry(ctx):
    lib, h = ctx
    for cap in (0, 1, 1000):
        want = _call(lib, h, "pgs_large_hits", *CASES[0], cap)
        got = _call(lib, h, "pgs_large_hits_static", *CASES[0], cap)
        assert got == want
        assert got[1] > cap  # the count is the total, not the written part


def test_static_rejects_cap_above_limit(ctx):
    lib, h = ctx
    rc = _call(lib, h, "pgs_large_hits_static", *CASES[1], STATIC_MAX + 1)[0]
    assert rc == pgsieve.PGS_EINVAL
    assert b"65536" in lib.pgs_last_error(h)
    # the limit itself is accepted
    assert _call(lib, h, "pgs_large_hits_static", *CASES[1], STATIC_MAX)[0] == pgsieve.PGS_OK


def test_static_rejects_invalid_prime_like_allocating_entry(ctx):
    lib, h = ctx
    bad = (1, 100, 5000, 20000, 3)  # prime <= 4*SL + 2
    assert _call(lib, h, "pgs_large_hits", *bad, 10)[0] == pgsieve.PGS_EINVAL
    assert _call(lib, h, "pgs_large_hits_static", *bad, 10)[0] == pgsieve.PGS_EINVAL
