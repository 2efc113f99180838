"""The device arithmetic (pg_arith.cuh), compiled for the host, against the oracle.

These are the exact functions the kernels run: the Euclid modulo search with
residue-tracking unwinding, the three-gap return structure, the chunked hit
enumeration that replaces modulo_search_euclid_all_large
(modulo_search.cpp:339-376), and the Montgomery K mod p.
"""
from __future__ import annotations

import ctypes
import random

import pytest

import pgo

_lib = None


@pytest.fixture(scope="module")
def ah(built):
    import build as pkg_build

    lib = ctypes.CDLL(str(pkg_build.ARITH_HOST_LIB))
    u64 = ctypes.c_uint64
    lib.ah_modsearch.restype = u64
    lib.ah_modsearch.argtypes = [u64, u64, u64, u64, ctypes.POINTER(u64)]
    lib.ah_three_gap.restype = None
    lib.ah_three_gap.argtypes = [u64, u64, u64, ctypes.POINTER(u64)]
    lib.ah_hits.restype = ctypes.c_size_t
    lib.ah_hits.argtypes = [u64, ctypes.c_uint32, ctypes.c_uint32, u64, u64, ctypes.c_uint32,
                            ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(u64), ctypes.c_size_t]
    lib.ah_hits_cf.restype = ctypes.c_size_t
    lib.ah_hits_cf.argtypes = lib.ah_hits.argtypes
    lib.ah_hits_items.restype = ctypes.c_size_t
    lib.ah_hits_items.argtypes = [u64, ctypes.c_uint32, ctypes.c_uint32, u64, u64, ctypes.c_uint32,
                                  ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32),
                                  ctypes.POINTER(u64), ctypes.c_size_t]
    lib.ah_hits_grid.restype = ctypes.c_size_t
    lib.ah_hits_grid.argtypes = [u64, ctypes.c_uint32, ctypes.c_uint32, u64, u64, u64, u64,
                                 ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(u64), ctypes.c_size_t]
    lib.ah_pow32_mod.restype = ctypes.c_uint32
    lib.ah_pow32_mod.argtypes = [ctypes.c_uint32, ctypes.c_int]
    lib.ah_return_walk_agrees.restype = ctypes.c_int
    lib.ah_return_walk_agrees.argtypes = [ctypes.c_uint32] * 9 + [ctypes.POINTER(ctypes.c_uint32), ctypes.c_size_t,
                                                                 ctypes.POINTER(ctypes.c_size_t)]
    lib.ah_udiv2f.restype = None
    lib.ah_udiv2f.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                              ctypes.POINTER(ctypes.c_uint32)]
    lib.ah_udiv2_64.restype = None
    lib.ah_udiv2_64.argtypes = [u64, u64, u64, ctypes.c_int, ctypes.POINTER(u64)]
    lib.ah_udiv2.restype = None
    lib.ah_udiv2.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                             ctypes.POINTER(ctypes.c_uint32)]
    lib.ah_first_entry.restype = None
    lib.ah_first_entry.argtypes = [u64, u64, u64, u64, ctypes.POINTER(u64)]
    lib.ah_first_entry_lim.restype = None
    lib.ah_first_entry_lim.argtypes = [u64, u64, u64, u64, u64, ctypes.POINTER(u64)]
    lib.ah_kmod.restype = u64
    lib.ah_kmod.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_int, u64]
    lib.ah_start32.restype = ctypes.c_uint32
    lib.ah_start32.argtypes = [ctypes.c_uint32, u64, ctypes.c_uint32, ctypes.c_uint32]
    lib.ah_mulmod.restype = u64
    lib.ah_mulmod.argtypes = [u64, u64, u64]
    return lib


def _hits(ah, M, max_mi, SL, p, r, chunk=0, cap=1 << 18, cf=False):
    mi = (ctypes.c_uint32 * cap)()
    md = (ctypes.c_uint64 * cap)()
    fn = ah.ah_hits_cf if cf else ah.ah_hits
    n = fn(M, max_mi, SL, p, r, chunk, mi, md, cap)
    assert n <= cap
    return list(zip(mi[:n], md[:n]))


def _rand_prime(rng, lo, hi):
    """A prime in [lo, hi) drawn from the seeded generator."""
    import sympy

    while True:
        q = sympy.nextprime(rng.randrange(lo, hi) - 1)
        if q < hi:
            return q


def test_modsearch_known_answers(ah):
    v = ctypes.c_uint64()
    assert ah.ah_modsearch(10**9 + 7, 123, 615, 621, ctypes.byref(v)) == 5
    assert v.value == 615
    assert ah.ah_modsearch(10**9 + 7, 123, 609, 615, ctypes.byref(v)) == 5


@pytest.mark.parametrize("bits", [20, 31, 32, 34, 40, 45])
def test_modsearch_vs_oracle(ah, bits):
    rng = random.Random(bits)
    v = ctypes.c_uint64()
    for _ in range(300):
        p = _rand_prime(rng, 2 ** (bits - 1), 2**bits)
        a = rng.randrange(1, p)
        width = rng.choice([0, 1, 5, 1000, 80000, p // 7])
        width = min(width, p - 2)
        l = rng.randrange(1, p - width)
        r = l + width
        k = ah.ah_modsearch(p, a, l, r, ctypes.byref(v))
        assert k == pgo.modulo_search(p, a, l, r)
        assert v.value == (k * a) % p
        assert l <= v.value <= r


def test_three_gap_brute(ah):
    rng = random.Random(7)
    out = (ctypes.c_uint64 * 4)()
    for _ in range(200):
        p = _rand_prime(rng, 1000, 200000)
        w = rng.randrange(2, p // 2 - 1)
        a = rng.randrange(1, p)
        ah.ah_three_gap(p, a, w, out)
        kp, up, kn, dn = list(out)
        # kp / kn: smallest k with k*a mod p in (0, w) / (p - w, p)
        k_up = next(k for k in range(1, p) if 0 < (k * a) % p < w)
        k_dn = next(k for k in range(1, p) if p - w < (k * a) % p < p)
        assert (kp, up) == (k_up, (k_up * a) % p)
        assert (kn, dn) == (k_dn, p - (k_dn * a) % p)
        assert up + dn >= w


@pytest.mark.parametrize("bits,chunk", [(18, 0), (18, 777), (24, 0), (24, 3000), (31, 0),
                                        (32, 0), (33, 0), (33, 50000), (36, 0), (40, 0)])
def test_hits_vs_all_large(ah, bits, chunk):
    """Every hit of modulo_search_euclid_all_large, in order, chunked or not."""
    rng = random.Random(bits * 1000 + chunk)
    for _ in range(60):
        SL = rng.choice([500, 4000, 20000, 40000])
        lo = max(4 * SL + 3, 2 ** (bits - 1))
        p = _rand_prime(rng, lo, max(2 * lo, 2**bits))
        r = rng.randrange(1, p)
        M = rng.randrange(1, 10**10)
        max_mi = rng.choice([1, 17, 1000, 100000])
        got = _hits(ah, M, max_mi, SL, p, r, chunk)
        want = pgo.all_large(M, max_mi, SL, p, r)
        assert got == want
        assert _hits(ah, M, max_mi, SL, p, r, chunk, cf=True) == want


def test_hits_dense_small_prime(ah):
    """p just above 4*SL+2: many hits per prime, exercising all three gaps."""
    rng = random.Random(3)
    for _ in range(20):
        SL = rng.choice([5000, 11000])
        p = _rand_prime(rng, 4 * SL + 3, 4 * SL + 2000)
        r = rng.randrange(1, p)
        M = rng.randrange(1, 10**9)
        got = _hits(ah, M, 50000, SL, p, r, 4096)
        want = pgo.all_large(M, 50000, SL, p, r)
        assert got == want
        assert _hits(ah, M, 50000, SL, p, r, 0, cf=True) == want


def _hits_items(ah, M, max_mi, SL, p, r, direct, item, cap=1 << 18):
    mi = (ctypes.c_uint32 * cap)()
    md = (ctypes.c_uint64 * cap)()
    n = ah.ah_hits_items(M, max_mi, SL, p, r, direct, item, mi, md, cap)
    assert n <= cap
    return list(zip(mi[:n], md[:n]))


@pytest.mark.parametrize("bits", [18, 24, 31, 32, 34, 40])
def test_hits_items_vs_all_large(ah, bits):
    """The kernel's split: direct walk or closed-form items of 64 (and odd sizes)."""
    rng = random.Random(bits + 77)
    for _ in range(80):
        SL = rng.choice([500, 4000, 20000, 40000])
        lo = max(4 * SL + 3, 2 ** (bits - 1))
        p = _rand_prime(rng, lo, max(2 * lo, 2**bits))
        r = rng.randrange(1, p)
        M = rng.randrange(1, 10**10)
        max_mi = rng.choice([1, 17, 1000, 100000])
        want = pgo.all_large(M, max_mi, SL, p, r)
        for direct, item in ((24, 64), (0, 64), (0, 7), (10**9, 64)):
            assert _hits_items(ah, M, max_mi, SL, p, r, direct, item) == want


@pytest.mark.parametrize("odd_d", [0, 1])
@pytest.mark.parametrize("bits", [18, 26, 31, 33, 40])
def test_parity_walk_vs_all_large(ah, bits, odd_d):
    """The parity-reduced walk yields exactly the hits with m*K + X odd."""
    ah.ah_hits_parity.restype = ctypes.c_size_t
    ah.ah_hits_parity.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                  ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32),
                                  ctypes.POINTER(ctypes.c_uint64), ctypes.c_size_t]
    rng = random.Random(bits * 10 + odd_d)
    cap = 1 << 18
    mi = (ctypes.c_uint32 * cap)()
    xs = (ctypes.c_uint64 * cap)()
    for _ in range(60):
        SL = rng.choice([500, 501, 4000, 4001, 20000, 40000])
        lo = max(4 * SL + 3, 2 ** (bits - 1))
        p = _rand_prime(rng, lo, max(2 * lo, 2**bits))
        r = rng.randrange(1, p)
        M = rng.randrange(1, 10**10)
        minc = rng.choice([1, 2, 17, 1000, 100000])
        n = ah.ah_hits_parity(M, minc, SL, p, r, odd_d, mi, xs, cap)
        got = sorted(zip(mi[:n], xs[:n]))
        want = []
        for m_i, t in pgo.all_large(M, minc, SL, p, r):
            x = 2 * SL - t
            X = x - SL
            m = M + m_i
            if odd_d:  # K even: m*K + X odd iff X odd
                ok = X % 2 == 1
            else:  # K odd, valid m odd: X even
                ok = m % 2 == 1 and X % 2 == 0
            if ok:
                want.append((m_i, x))
        assert got == sorted(want), (SL, p, r, M, minc)


def test_first_entry_brute(ah):
    """First k >= 0 with (y0 + k*a) mod p < w, and the three-gap data, by brute force."""
    rng = random.Random(13)
    out = (ctypes.c_uint64 * 6)()
    for _ in range(400):
        p = _rand_prime(rng, 50, 60000)
        w = rng.randrange(2, (p - 1) // 2)  # the sieve's window is 2*SL+1 >= 3
        a = rng.randrange(1, p)
        y0 = rng.randrange(0, p)
        ah.ah_first_entry(p, a, w, y0, out)
        t, y, kp, up, kn, dn = list(out)
        k = next(k for k in range(0, p) if (y0 + k * a) % p < w)
        assert (t, y) == (k, (y0 + k * a) % p), (p, a, w, y0)
        k_up = next(k for k in range(1, p) if 0 < (k * a) % p < w)
        k_dn = next(k for k in range(1, p) if p - w < (k * a) % p < p)
        assert (kp, up, kn, dn) == (k_up, (k_up * a) % p, k_dn, p - (k_dn * a) % p)


def test_first_entry_early_stop(ah):
    """With t_lim, the search either returns the full answer (first hit below
    t_lim) or stops with t >= t_lim exactly when the first hit is >= t_lim."""
    rng = random.Random(19)
    full = (ctypes.c_uint64 * 6)()
    lim = (ctypes.c_uint64 * 6)()
    stopped = 0
    for _ in range(3000):
        bits = rng.choice([16, 24, 31, 32, 40, 45])
        p = _rand_prime(rng, 2 ** (bits - 1), 2 ** bits)
        w = rng.choice([3, 101, 2001, 20001, 40001])
        if w >= p // 2:
            continue
        a = rng.randrange(1, p)
        y0 = rng.randrange(0, p)
        ah.ah_first_entry(p, a, w, y0, full)
        t_true = full[0]
        t_lim = rng.choice([0, 1, t_true, t_true + 1, rng.randrange(0, 2 * t_true + 2), 2**64 - 1])
        ah.ah_first_entry_lim(p, a, w, y0, t_lim, lim)
        if t_true < t_lim:
            assert list(lim) == list(full), (p, a, w, y0, t_lim)
        else:
            assert lim[0] >= t_lim, (p, a, w, y0, t_lim)
            stopped += 1
    assert stopped > 500


def test_first_entry_wide(ah):
    """64-bit moduli against the oracle's Euclid search."""
    rng = random.Random(17)
    out = (ctypes.c_uint64 * 6)()
    for _ in range(300):
        p = _rand_prime(rng, 2**33, 2**45)
        w = rng.choice([1001, 40001, 80001])
        a = rng.randrange(1, p)
        y0 = rng.randrange(w, p)
        ah.ah_first_entry(p, a, w, y0, out)
        t, y = out[0], out[1]
        # smallest k >= 1 with k*a mod p in [p - y0, p - y0 + w - 1]
        k = pgo.modulo_search(p, a, p - y0, p - y0 + w - 1)
        assert (t, y) == (k, (y0 + k * a) % p)


@pytest.mark.parametrize("P,d", [(503, 210), (907, 2190), (1511, 2190), (3001, 2190), (953, 1)])
def test_kmod_vs_oracle(ah, P, d):
    limbs = pgo.build_k(P, d)
    arr = (ctypes.c_uint32 * len(limbs))(*limbs)
    rng = random.Random(P)
    qs = pgo.primes(P + 1, P + 3000)[:50]
    qs += [_rand_prime(rng, 2**30, 2**31) for _ in range(20)]
    qs += [_rand_prime(rng, 2**31, 2**32) for _ in range(20)]
    qs += [_rand_prime(rng, 2**32, 2**45) for _ in range(40)]
    for q in qs:
        assert ah.ah_kmod(arr, len(limbs), q) == pgo.k_mod(limbs, q)


def test_kmod4_interleaved(ah):
    ah.ah_kmod4.restype = None
    ah.ah_kmod4.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_int,
                            ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]
    rng = random.Random(21)
    for P, d in [(503, 210), (1511, 2190)]:
        limbs = pgo.build_k(P, d)
        arr = (ctypes.c_uint32 * len(limbs))(*limbs)
        for lo, hi in [(P + 1, 10**5), (2**30, 2**31), (2**31, 2**32)]:
            for _ in range(20):
                qs = [_rand_prime(rng, lo, hi) for _ in range(4)]
                out = (ctypes.c_uint32 * 4)()
                ah.ah_kmod4(arr, len(limbs), (ctypes.c_uint32 * 4)(*qs), out)
                assert list(out) == [pgo.k_mod(limbs, q) for q in qs]


def test_kmod_lsb_vs_oracle(ah):
    """Least-significant-limb-first chains (32-bit x4 and 64-bit words)."""
    u32p = ctypes.POINTER(ctypes.c_uint32)
    ah.ah_kmod4_lsb.restype = None
    ah.ah_kmod4_lsb.argtypes = [u32p, ctypes.c_int, u32p, u32p, u32p]
    ah.ah_kmod64_lsb.restype = ctypes.c_uint64
    ah.ah_kmod64_lsb.argtypes = [u32p, ctypes.c_int, ctypes.c_uint64]
    rng = random.Random(23)
    for P, d in [(503, 210), (1009, 1), (1511, 2190), (3001, 2190), (3001, 30030), (7, 7)]:
        limbs = pgo.build_k(P, d)
        arr = (ctypes.c_uint32 * len(limbs))(*limbs)
        for lo, hi in [(P + 1, 10**5), (2**30, 2**31), (2**31, 2**32 - 5)]:
            for _ in range(15):
                qs = [_rand_prime(rng, max(lo, 3), hi) for _ in range(4)]
                out = (ctypes.c_uint32 * 4)()
                r2 = (ctypes.c_uint32 * 4)()
                ah.ah_kmod4_lsb(arr, len(limbs), (ctypes.c_uint32 * 4)(*qs), out, r2)
                assert list(out) == [pgo.k_mod(limbs, q) for q in qs], (P, d, qs)
                assert list(r2) == [pow(2, 64, q) for q in qs]
        for q in [4294967291] + [_rand_prime(rng, 2**32, 2**46) for _ in range(30)]:
            assert ah.ah_kmod64_lsb(arr, len(limbs), q) == pgo.k_mod(limbs, q), (P, d, q)
        # odd limb counts and the largest 32-bit prime
        out = (ctypes.c_uint32 * 4)()
        r2 = (ctypes.c_uint32 * 4)()
        qs = [4294967291, 4294967279, 3, 5]
        ah.ah_kmod4_lsb(arr, len(limbs), (ctypes.c_uint32 * 4)(*qs), out, r2)
        assert list(out) == [pgo.k_mod(limbs, q) for q in qs]


def test_kmod_against_python_bignum(built):
    from sympy import primorial

    for P, d in [(503, 210), (3001, 2190)]:
        K = primorial(P, nth=False) // d
        limbs = pgo.build_k(P, d)
        assert sum(l << (32 * i) for i, l in enumerate(limbs)) == K


def test_start32(ah):
    rng = random.Random(11)
    for _ in range(500):
        p = _rand_prime(rng, 3, 2**32)
        r = rng.randrange(0, p)
        M = rng.randrange(1, 10**10 + 1)
        sl = rng.randrange(0, min(p, 100000))
        assert ah.ah_start32(r, M, sl, p) == (r * M + sl) % p


def test_redc32_and_inverse(ah):
    """REDC for R = 2^32 over the whole 32-bit prime range, including the
    largest moduli, where the reduced sum passes 2^32 before its one
    subtraction, and inputs up to p * 2^32 - 1."""
    ah.ah_redc32.restype = ctypes.c_uint32
    ah.ah_redc32.argtypes = [ctypes.c_uint64, ctypes.c_uint32]
    ah.ah_neg_inv32.restype = ctypes.c_uint32
    ah.ah_neg_inv32.argtypes = [ctypes.c_uint32]
    rng = random.Random(41)
    moduli = [3, 5, 7, 65537, 2**31 - 1, 2**31 + 11, 2**32 - 5, 2**32 - 17]
    moduli += [rng.randrange(3, 2**32 - 4) | 1 for _ in range(300)]
    for p in moduli:
        assert (p * ah.ah_neg_inv32(p)) % 2**32 == 2**32 - 1
        rinv = pow(2**32, -1, p)
        tops = [p * 2**32 - 1, p * 2**32 - 2**32, (p - 1) * 2**32 + 1, 0, 1]
        for t in tops + [rng.randrange(0, p * 2**32) for _ in range(40)]:
            assert ah.ah_redc32(t, p) == t * rinv % p, (t, p)


def test_walk_start(ah):
    """Step and start residue of the parity-reduced walk (32- and 64-bit)."""
    ah.ah_walk_start.restype = None
    ah.ah_walk_start.argtypes = [ctypes.c_uint64] * 3 + [ctypes.c_uint32] * 2 + [ctypes.POINTER(ctypes.c_uint64)]
    rng = random.Random(29)
    out = (ctypes.c_uint64 * 2)()
    for _ in range(1500):
        p = _rand_prime(rng, 3, rng.choice([2**20, 2**32 - 5, 2**46]))
        r = rng.randrange(0, p)
        m0 = rng.randrange(1, 10**10 + 1)
        c_add = rng.randrange(0, min(p // 8 + 1, 50000))
        odd = rng.randrange(2)
        ah.ah_walk_start(p, r, m0, c_add, odd, out)
        rh = r * pow(2, -1, p) % p
        c = c_add + ((p + 1) // 2 if odd else 0)
        assert list(out) == [rh if odd else r, (rh * m0 + c) % p], (p, r, m0, c_add, odd)


def test_mulmod(ah):
    rng = random.Random(5)
    for _ in range(1000):
        p = _rand_prime(rng, 3, 2**46)
        a, b = rng.randrange(p), rng.randrange(p)
        assert ah.ah_mulmod(a, b, p) == a * b % p


@pytest.mark.parametrize("threads,cta,cap", [(1, 1, 1 << 16), (155648, 256, 1 << 16), (7, 3, 1000), (1000, 256, 1),
                                             (64, 256, 0)])
def test_hits_grid_split_vs_oracle(ah, threads, cta, cap):
    """pgs_large_hits' grid form: the total over runs of steps started from
    the closed form, and the first cap hits written in order from the first
    2*cap + 2 steps, against the reference enumeration (18- to 45-bit primes,
    window up to 2e4)."""
    rng = random.Random(77 + threads + cap)
    cases = [(1234567, 100000, 5000, 20011, 7919)]
    for bits in (18, 25, 31, 33, 40, 45):
        for q in pgo.primes(2 ** (bits - 1), 2 ** (bits - 1) + 3000)[:3]:
            SL = rng.choice([1000, 5000, 20000])
            if q <= 4 * SL + 2:
                continue
            cases.append((rng.randrange(1, 10**9), rng.choice([1, 999, 100000, 3000000]), SL, q,
                          rng.randrange(1, q)))
    for M, max_mi, SL, q, r in cases:
        want = pgo.all_large(M, max_mi, SL, q, r, cap=1 << 22)
        mi = (ctypes.c_uint32 * max(1, cap))()
        md = (ctypes.c_uint64 * max(1, cap))()
        n = ah.ah_hits_grid(M, max_mi, SL, q, r, threads, cta, mi, md, cap)
        k = min(n, cap)
        assert n == len(want), (M, max_mi, SL, q, r)
        assert list(zip(mi[:k], md[:k])) == [tuple(h) for h in want[:k]], (M, max_mi, SL, q, r)


def test_return_walk_equals_circle_walk(ah):
    """The hit-to-hit walk (three-gap first-return map) emits exactly the
    circle walk's hits, in order, for any start on the circle (a hit or a
    miss), any step budget (items of the rotation, budgets ending on the
    middle of a two-step return) and any mi bound."""
    rng = random.Random(23)
    cap = 1 << 16
    buf = (ctypes.c_uint32 * cap)()
    n = ctypes.c_size_t()
    total = 0
    for _ in range(3000):
        bits = rng.choice([13, 21, 29, 32])
        p = _rand_prime(rng, 2 ** (bits - 1), 2 ** bits)
        w = rng.randrange(3, max(4, min(p // 2 - 1, 1 << 16)))
        if 2 * w >= p:
            continue
        a = rng.randrange(1, p)
        out = (ctypes.c_uint64 * 6)()
        ah.ah_first_entry(p, a, w, rng.randrange(0, p), out)
        _, _, kp, up, kn, dn = list(out)
        C = up + dn
        mi_hi = rng.choice([1, 7, 1000, 50000, 1 << 30])
        steps = rng.choice([1, 2, 3, 24, 64, 1000])
        kp32, kn32 = min(kp, mi_hi), min(kn, mi_hi)
        y = rng.randrange(0, C)
        mi = rng.randrange(0, mi_hi)
        ok = ah.ah_return_walk_agrees(mi, y, kp32, up, kn32, dn, w, mi_hi, steps, buf, cap, ctypes.byref(n))
        assert ok == 1, (p, a, w, mi, y, mi_hi, steps)
        total += n.value
    assert total > 10000


def test_udiv2_shared_reciprocal_exact(ah):
    """The continued fraction's two quotients by one reciprocal equal the
    exact quotients for every divisor size, small and large quotients (the
    fast path and the fallback), with the reciprocal moved up to 2 ulps
    either way (the device's rcp.approx is within 1 ulp)."""
    rng = random.Random(3)
    out = (ctypes.c_uint32 * 2)()
    cases = []
    for _ in range(40000):
        d = rng.choice([1, 2, 3, rng.randrange(1, 1 << 8), rng.randrange(1, 1 << 16), rng.randrange(1, 1 << 24),
                        rng.randrange(1, 1 << 32), (1 << 32) - 1, (1 << 24) + 1, (1 << 31) + 1])
        qmax = rng.choice([3, 1 << 10, 1 << 17, 1 << 18, 1 << 32])
        def num():
            v = rng.randrange(0, qmax) * d + rng.randrange(0, d)
            return v if v < (1 << 32) else rng.randrange(0, 1 << 32)
        cases.append((num(), num(), d))
    # quotients right at the fast-path edge and exact multiples
    for d in (1, 2, 7, 1000003, 65537):
        for q in ((1 << 17) - 1, 1 << 17, (1 << 17) + 1, (1 << 18) - 1):
            for dr in (0, d - 1):
                n = q * d + dr
                if n < (1 << 32):
                    cases.append((n, n, d))
    for n1, n2, d in cases:
        for skew in (-2, -1, 0, 1, 2):
            ah.ah_udiv2(n1, n2, d, skew, out)
            assert (out[0], out[1]) == (n1 // d, n2 // d), (n1, n2, d, skew)
            ah.ah_udiv2f(n1, n2, d, skew, out)
            assert (out[0], out[1]) == (n1 // d, n2 // d), ("f", n1, n2, d, skew)


def test_udiv2_64_shared_reciprocal_exact(ah):
    """The 64-bit continued fraction's two quotients by one single-precision
    reciprocal equal the exact quotients: divisors up to 2^64, quotients on
    both sides of the fast-path edge (2^17), the reciprocal moved up to 2 ulps
    either way."""
    rng = random.Random(5)
    out = (ctypes.c_uint64 * 2)()
    cases = []
    for _ in range(30000):
        d = rng.choice([1, 2, 3, rng.randrange(1, 1 << 16), rng.randrange(1, 1 << 33), rng.randrange(1, 1 << 46),
                        rng.randrange(1, 1 << 64), (1 << 46) - 1, (1 << 24) + 1, (1 << 40) + 1, (1 << 64) - 1])
        qmax = rng.choice([3, 1 << 10, 1 << 17, 1 << 18, 1 << 40, 1 << 64])
        def num():
            v = rng.randrange(0, qmax) * d + rng.randrange(0, d)
            return v if v < (1 << 64) else rng.randrange(0, 1 << 64)
        cases.append((num(), num(), d))
    for d in (1, 3, 1000003, (1 << 33) + 17, (1 << 45) + 59):
        for q in ((1 << 17) - 1, 1 << 17, (1 << 17) + 1, (1 << 18) - 1, (1 << 18) + 1):
            for dr in (0, d - 1):
                n = q * d + dr
                if n < (1 << 64):
                    cases.append((n, n, d))
    for n1, n2, d in cases:
        for skew in (-2, -1, 0, 1, 2):
            ah.ah_udiv2_64(n1, n2, d, skew, out)
            assert (out[0], out[1]) == (n1 // d, n2 // d), (n1, n2, d, skew)


def test_pow64_128_and_inverse_without_division(ah):
    """2^64 and 2^128 mod p (eight single-precision reduction steps, the
    reciprocal skewed up to 2 ulps) and -p^-1 mod 2^64 for odd p up to 2^46,
    the 64-bit primes' K mod p set-up."""
    ah.ah_pow64_128.restype = None
    ah.ah_pow64_128.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
    ah.ah_neg_inv64.restype = ctypes.c_uint64
    ah.ah_neg_inv64.argtypes = [ctypes.c_uint64]
    rng = random.Random(31)
    ps = [3, 5, 65537, (1 << 31) - 1, (1 << 32) + 15, (1 << 46) - 1, (1 << 45) + 1]
    ps += [rng.randrange(3, 1 << b) | 1 for b in (8, 17, 24, 32, 33, 40, 46) for _ in range(500)]
    out = (ctypes.c_uint64 * 2)()
    for p in ps:
        for skew in (-2, 0, 2):
            ah.ah_pow64_128(p, skew, out)
            assert (out[0], out[1]) == (pow(2, 64, p), pow(2, 128, p)), (p, skew)
        assert (ah.ah_neg_inv64(p) * p) % (1 << 64) == (1 << 64) - 1, p


def test_pow32_mod_without_division(ah):
    """2^32 mod p of the K mod p setup (reciprocal and two subtractions) for
    odd p across the three ranges and their edges, reciprocal skewed up to
    2 ulps either way."""
    rng = random.Random(8)
    ps = [3, 5, 65535, 65537, 65539, (1 << 31) - 1, (1 << 31) + 1, (1 << 32) - 5, (1 << 32) - 1]
    ps += [rng.randrange(1, 1 << b) | 1 for b in (17, 20, 24, 28, 31, 32) for _ in range(3000)]
    for p in ps:
        for skew in (-2, 0, 2):
            assert ah.ah_pow32_mod(p, skew) == (1 << 32) % p, (p, skew)
