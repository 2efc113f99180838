"""Pin the CPU oracle against the reference's own golden vectors.

The md5 values come from misc/tests.sh:66-94 and EXTENDED.md:186-187 of the
reference, plus reference runs recorded by tests/golden/make_goldens.py.  The
modulo-search known answers are misc/modulo_check.py:126-143.
"""
from __future__ import annotations

import hashlib

import pytest

import pgo

FAST = ["fn1", "fn1_rle", "fn1_bitcompressed", "fn2", "config1", "small_d1", "small_d2",
        "small_d30", "small_d2190", "small_d30030", "small_d7_odd", "small_d73_sl_odd",
        "small_rle_d210", "small_bc_d30", "edge_maxprime_1M",
        # m past 2^32, up to the reference's mstart + minc <= 1e10 + 1
        "big_m_cross_2e32", "big_m_1e10_d7_odd", "big_m_rle_d2190", "big_m_bc_d30"]


def _job(g):
    return dict(p=g["p"], d=g["d"], mstart=g["mstart"], minc=g["minc"], sieve_length=g["sieve_length"],
                max_prime=g["max_prime"], compression=g["compression"])


@pytest.mark.parametrize("name", FAST)
def test_oracle_matches_reference_md5(built, goldens, name):
    g = goldens[name]
    data = pgo.method2(**_job(g), threads=8)
    assert len(data) == g["bytes"]
    assert hashlib.md5(data).hexdigest() == g["md5"]


@pytest.mark.slow
def test_oracle_extended_1e9(built, goldens):
    g = goldens["ext_907_210"]
    data = pgo.method2(**_job(g), threads=8)
    assert hashlib.md5(data).hexdigest() == g["md5"] == "d74bd47c8d43eac9a2309fc7722839ac"


def test_published_md5_values(goldens):
    # values printed in the reference's own tests
    assert goldens["fn1"]["md5"] == "15a5cbff7301262caf047028c05f0525"
    assert goldens["fn1_rle"]["md5"] == "2ed7b0b9621dab602f204865360a3c56"
    assert goldens["fn1_bitcompressed"]["md5"] == "6edd5f50c4f588890a168461a7240c47"
    assert goldens["fn2"]["md5"] == "a8d85c965ddf2d9601e93c9920a9aa12"


def test_modulo_search_known_answers(built):
    # misc/modulo_check.py:128-133
    assert pgo.modulo_search(10**9 + 7, 123, 5 * 123, 5 * 123 + 6) == 5
    assert pgo.modulo_search(10**9 + 7, 123, 5 * 123 - 6, 5 * 123) == 5
    # misc/modulo_check.py:136-143: last 100 primes below 1e5
    ps = pgo.primes(10**4, 10**5)[-100:]
    assert len(ps) == 100
    assert sum(pgo.modulo_search(p, 123, 1000, 1010) for p in ps) == 780012
    assert sum(pgo.modulo_search_stack(p, 123, 1000, 1010) for p in ps) == 780012


def test_oracle_primes_count(built):
    # pi(10^7) = 664579 (gap_common.cpp:45)
    assert len(pgo.primes(0, 10**7)) == 664579


def test_trial_division_definition(built, goldens):
    """Surviving offsets have no factor below the sieve limit; removed ones do."""
    g = goldens["fn1"]
    job = {k: g[k] for k in ("p", "d", "mstart", "minc", "sieve_length", "max_prime")}
    text = pgo.method2(**job).decode()
    ms, xs, expect_prime = [], [], []
    for line in text.splitlines()[:6]:
        head, low, high = line.split("|")
        m = int(head.split(":")[0])
        lows = [-int(v[1:]) for v in low.split()]
        highs = [int(v[1:]) for v in high.split()]
        for x in lows[:3] + highs[:3]:
            ms.append(m)
            xs.append(x)
            expect_prime.append(True)
        # a removed offset: odd X makes m*K + X even for this odd-K (d even) job
        ms.append(m)
        xs.append(1)
        expect_prime.append(False)
    f = pgo.trial_division(job, ms, xs)
    for factor, ok in zip(f, expect_prime):
        assert (factor == 0) == ok
