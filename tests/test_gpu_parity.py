"""Parity of the CUDA path with the oracle and the reference's golden files.

Every unknowns file produced on the GPU must be byte-identical to the
reference's (md5 from tests/golden/goldens.json) and to the CPU oracle.
"""
from __future__ import annotations

import hashlib
import random

import pytest

import pgo
import pgsieve

pytestmark = pytest.mark.gpu

GOLDEN_NAMES = ["fn1", "fn1_rle", "fn1_bitcompressed", "small_bc_d30", "fn2", "config1", "small_d1", "small_d2", "small_d30",
                "small_d2190", "small_d30030", "small_d7_odd", "small_d73_sl_odd",
                "small_rle_d210", "edge_maxprime_1M", "ext_907_210",
                # m past 2^32, up to the reference's mstart + minc <= 1e10 + 1
                "big_m_cross_2e32", "big_m_1e10_d7_odd", "big_m_rle_d2190", "big_m_bc_d30"]


def _spec(g) -> pgsieve.JobSpec:
    return pgsieve.JobSpec(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"],
                           g["max_prime"], g["compression"])


def _first_diff(a: bytes, b: bytes) -> str:
    la, lb = a.split(b"\n"), b.split(b"\n")
    for i, (x, y) in enumerate(zip(la, lb)):
        if x != y:
            return f"row {i}: gpu={x[:200]!r} want={y[:200]!r}"
    return f"row count gpu={len(la)} want={len(lb)}"


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_method2_matches_reference_golden(sieve, goldens, name):
    g = goldens[name]
    data = sieve.method2(_spec(g))
    if hashlib.md5(data).hexdigest() != g["md5"]:
        want = pgo.method2(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"],
                           g["max_prime"], g["compression"], threads=16)
        pytest.fail(f"{name}: md5 mismatch; {_first_diff(data, want)}")
    assert len(data) == g["bytes"]


def test_config2_full_size_matches_reference(sieve, goldens):
    """Config 2 (P=1511, d=2190, minc=1e5, SL=2e4, max_prime=2e9)."""
    g = goldens["config2"]
    data = sieve.method2(_spec(g))
    assert hashlib.md5(data).hexdigest() == g["md5"]


def test_config3_full_size_matches_reference(sieve, goldens):
    """Config 3 (P=3001, d=2190, minc=1e5, SL=4e4, max_prime=1e10): 2.52e8 of
    its 4.55e8 primes lie above 2^32 (64-bit K mod p and walk starts).  The
    golden is the reference's --method1 file (its method2 aborts on this job,
    combined_sieve.cpp:1229; the two methods write the same bytes)."""
    g = goldens["config3"]
    data = sieve.method2(_spec(g))
    assert hashlib.md5(data).hexdigest() == g["md5"]
    assert len(data) == g["bytes"]


def _random_jobs(n, seed):
    rng = random.Random(seed)
    jobs = []
    while len(jobs) < n:
        P = rng.choice([503, 509, 521, 601, 797, 907, 1009])
        d = rng.choice([1, 2, 3, 6, 7, 30, 210, 2190 if P >= 73 else 210, 30030, 46])
        if d % 4 == 0:
            continue
        SL = rng.randrange(6 * P // 500 + 1, 22 * P // 500 + 1) * 500
        minc = rng.choice([1, 7, 100, 1000, 3000])
        mstart = rng.randrange(1, 10**9)
        max_prime = rng.choice([1, 3, 10, 40]) * 1_000_000
        comp = rng.choice([0, 0, 1, 2])
        jobs.append((P, d, mstart, minc, SL, max_prime, comp))
    return jobs


@pytest.mark.parametrize("job", _random_jobs(24, 2024))
def test_method2_random_vs_oracle(sieve, job):
    P, d, mstart, minc, SL, mp, comp = job
    spec = pgsieve.JobSpec(P, d, mstart, minc, SL, mp, comp)
    pl = pgsieve.plan(spec)
    if pl["rc"] != 0:
        pytest.skip(f"reference rejects this job ({pl['rc']})")
    got = sieve.method2(spec)
    want = pgo.method2(P, d, mstart, minc, SL, mp, comp, threads=16)
    assert got == want, _first_diff(got, want)


@pytest.mark.parametrize("minc", [177_000, 340_000, 400_000])
def test_method2_masks_near_shared_memory_limits(sieve, minc):
    """Valid-m and live-offset masks (8 bytes per 32 walk indices or
    residues; odd d walks every m) whose shared-memory copy, together with the
    large kernel's static shared memory, crosses the 48 KiB default (177,000
    m: 44.5 KiB), nears the 96 KiB limit of the shared copy (340,000 m: 83.3
    KiB) or exceeds it and is read from global memory (400,000 m: 97.9 KiB)."""
    spec = pgsieve.JobSpec(89, 105, 1000003, minc, 1000, 2_000_000, 1)
    got = sieve.method2(spec)
    want = pgo.method2(89, 105, 1000003, minc, 1000, 2_000_000, 1, threads=16)
    assert got == want, _first_diff(got, want)


@pytest.mark.parametrize("name", ["fn1", "config1", "small_bc_d30", "small_rle_d210"])
def test_method2_text_pipeline_short_estimate(sieve, goldens, name, monkeypatch):
    """The one-call path copies each chunk of rows' text to the host while
    later chunks run, into a buffer sized from the first chunk; with the
    estimate cut to 5 % every later chunk overruns it and the text moves to
    an exact buffer part way.  The bytes must not change."""
    monkeypatch.setenv("PGSIEVE_TEXT_ESTIMATE", "0.05")
    g = goldens[name]
    data = sieve.method2(_spec(g))
    assert hashlib.md5(data).hexdigest() == g["md5"]
    assert len(data) == g["bytes"]


@pytest.mark.parametrize("name", ["fn1", "fn1_rle", "fn1_bitcompressed", "small_d7_odd"])
def test_result_unknowns_count(sieve, goldens, name):
    """pgs_result.unknowns is the number of unknown offsets in the file: the
    header counts of the plain text, whatever the compression."""
    g = goldens[name]
    st: dict = {}
    with sieve.prepare(_spec(g)) as prep:
        prep.run(False)
        prep.fetch(st)
    plain = pgo.method2(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"], 0,
                        threads=16).decode()
    total = 0
    for line in plain.splitlines():
        head = line.split("|")[0].split(":")[1].split()
        total += -int(head[0]) + int(head[1])
    assert st["unknowns"] == total


def test_prepare_run_fetch_repeatable(sieve, goldens):
    g = goldens["fn1"]
    with sieve.prepare(_spec(g)) as prep:
        outs = []
        for _ in range(3):
            prep.run()
            outs.append(prep.fetch())
    assert all(hashlib.md5(o).hexdigest() == g["md5"] for o in outs)


def test_primes_vs_oracle(sieve):
    # segments wholly below 2^32 take 32-bit remainders (the last of them ends
    # just below 2^32); segments reaching past it take 64-bit ones
    for lo, hi in [(0, 100), (0, 10**6), (10**9, 10**9 + 10**6), (2**32 - 2 * 10**6, 2**32 - 1),
                   (2**32 - 10**5, 2**32 + 10**5), (10**10, 10**10 + 3 * 10**5)]:
        assert sieve.primes(lo, hi) == pgo.primes(lo, hi), (lo, hi)


def test_prime_count_1e9(sieve):
    # pi(1e9) = 50,847,534 (gap_common.cpp:51)
    assert len(sieve.primes(0, 10**9)) == 50847534


def test_k_mod_p_vs_oracle(sieve):
    rng = random.Random(9)
    for P, d in [(503, 210), (1511, 2190), (3001, 2190)]:
        limbs = pgo.build_k(P, d)
        qs = pgo.primes(P + 1, P + 5000)[:200]
        qs += [q for q in pgo.primes(2**31 - 10**4, 2**31 + 10**4)]
        qs += [q for q in pgo.primes(2**33, 2**33 + 10**4)][:100]
        qs += [q for q in pgo.primes(3 * 10**13, 3 * 10**13 + 3000)]
        rng.shuffle(qs)
        got = sieve.k_mod_p(limbs, qs)
        assert got == [pgo.k_mod(limbs, q) for q in qs]


def test_modulo_search_vs_oracle(sieve):
    rng = random.Random(4)
    P, A, L, R = [], [], [], []
    for bits in (20, 32, 34, 45):
        for q in pgo.primes(2 ** (bits - 1), 2 ** (bits - 1) + 20000)[:200]:
            a = rng.randrange(1, q)
            w = rng.choice([0, 10, 80000])
            l = rng.randrange(1, q - w)
            P.append(q), A.append(a), L.append(l), R.append(l + w)
    got = sieve.modulo_search(P, A, L, R)
    assert got == [pgo.modulo_search(*t) for t in zip(P, A, L, R)]


def test_large_hits_vs_oracle(sieve):
    rng = random.Random(5)
    for bits in (20, 31, 34):
        for q in pgo.primes(2 ** (bits - 1), 2 ** (bits - 1) + 5000)[:10]:
            SL = 5000
            if q <= 4 * SL + 2:
                continue
            r = rng.randrange(1, q)
            M = rng.randrange(1, 10**9)
            got = sieve.large_hits(M, 100000, SL, q, r)
            assert got == pgo.all_large(M, 100000, SL, q, r)
