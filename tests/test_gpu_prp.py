"""Device probable-prime tests and gap search against the oracle and the
reference's own gap_test_simple runs (tests/golden/gaps.json)."""
from __future__ import annotations

import json
import random
from pathlib import Path

import pytest

import pgsieve
import prp_oracle as po

pytestmark = pytest.mark.gpu

GAPS = json.loads((Path(__file__).resolve().parent / "golden" / "gaps.json").read_text())

MERSENNE_EXP = [61, 89, 107, 127, 521, 607, 1279, 2203, 2281, 3217]


def _odd(rng, bits):
    return rng.getrandbits(bits) | (1 << (bits - 1)) | 1


def test_prp_small_numbers_and_pseudoprimes(sieve):
    nums = list(range(0, 3000)) + [2047, 3277, 4033, 4681, 8321, 15841, 29341, 561, 1105, 1729]
    got = sieve.prp_test(nums)
    for n, g in zip(nums, got):
        want = n in (2, 3, 5, 7) if n < 8 else (n % 2 == 1 and po.strong_prp2(n))
        assert g == want, n


@pytest.mark.parametrize("bits", [40, 200, 252, 253, 300, 600, 1000, 1293, 1600, 2100, 2160, 2300, 2600, 3100,
                                  3600, 4092])
def test_prp_random_numbers_every_width(sieve, bits):
    """Each batch's largest number sets the limbs per lane (1..16): a batch per
    width, random odd numbers, products of two primes and primes."""
    rng = random.Random(bits)
    nums = [_odd(rng, bits) for _ in range(24)]
    # numbers with long runs of trailing zeros in N - 1 (large s)
    t = max(2, bits // 3)
    nums += [(_odd(rng, bits - t) << t) + 1, (1 << (bits - 1)) + 1]
    got = sieve.prp_test(nums)
    assert got == [po.strong_prp2(n) for n in nums]
    # probable primes (the next one above a random start, found by the oracle;
    # wider primes are the Mersenne primes below) and a multiple of one
    if bits <= 1100:
        x = _odd(rng, bits - 2)
        while not po.strong_prp2(x):
            x += 2
        assert sieve.prp_test([x, x + 2, 3 * x]) == [True, po.strong_prp2(x + 2), False]


def test_prp_mersenne_primes_and_composites(sieve):
    nums = [(1 << e) - 1 for e in MERSENNE_EXP] + [(1 << 1277) - 1, (1 << 2203) + 1, (1 << 3217) - 3]
    want = [True] * len(MERSENNE_EXP) + [po.strong_prp2(n) for n in nums[len(MERSENNE_EXP):]]
    assert sieve.prp_test(nums) == want


def test_prp_rejects_too_wide(sieve):
    with pytest.raises(pgsieve.PgsError) as ei:
        sieve.prp_test([(1 << 4093) - 1])
    assert ei.value.code == pgsieve.PGS_EINVAL


def _lists(sieve, g):
    job = pgsieve.JobSpec(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"],
                          g["compression"])
    return sieve.parse_unknowns(job, sieve.method2(job))


@pytest.mark.parametrize("name", sorted(GAPS))
def test_prp_gaps_match_reference_gap_test(sieve, name):
    """Sieve on the device, parse on the device, gap search on the device:
    every (m, prev, next) and the total PRP test count as the reference's
    gap_test_simple (both sides, GMP's primality test, prevprime / nextprime
    past the sieve length)."""
    g = GAPS[name]
    lists = _lists(sieve, g)
    res, stats = sieve.prp_gaps(g["p"], g["d"], g["sieve_length"], lists)
    got = [[int(lists["m"][i]), r[0], r[1]] for i, r in enumerate(res)]
    assert got == g["gaps"]
    assert sum(r[2] + r[3] for r in res) == g["prp_tests"]
    sl = g["sieve_length"]
    assert sum(1 for r in res if r[4] & 1) + sum(1 for r in res if r[4] & 2) == g["past_sieve_length"]
    assert all(bool(r[4] & 1) == (r[0] > sl) and bool(r[4] & 2) == (r[1] > sl) for r in res)
    assert stats["prp_tests"] >= g["prp_tests"] and stats["rounds"] > 0


@pytest.mark.parametrize("name", sorted(GAPS))
def test_prp_gaps_on_prepared_job_in_place(sieve, name):
    """pgs_prp_gaps_prepared: the same gaps from the job's device lists,
    without the lists leaving the device."""
    g = GAPS[name]
    job = pgsieve.JobSpec(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"],
                          g["compression"])
    with sieve.prepare(job) as prep:
        prep.run(False)
        res, _ = prep.prp_gaps()
        m = prep.unknowns()["m"]
    assert [[int(m[i]), r[0], r[1]] for i, r in enumerate(res)] == g["gaps"]
    assert sum(r[2] + r[3] for r in res) == g["prp_tests"]


def test_prp_gaps_one_side_skip_matches_oracle(sieve):
    g = GAPS["small_bc_d30"]
    lists = _lists(sieve, g)
    k = po.primorial_k(g["p"], g["d"])
    res, _ = sieve.prp_gaps(g["p"], g["d"], g["sieve_length"], lists, min_merit=5.0, one_side_skip=True)
    want = po.gap_search(k, g["sieve_length"], lists, min_merit=5.0, one_side_skip=True)
    assert res == want
    skipped = sum(1 for r in res if r[4] & 4)
    assert 0 < skipped < len(res)


def test_prp_gaps_rejects_bad_input(sieve):
    lists = {"m": [5], "start": [0], "n_prev": [3], "n_next": [0], "dist": [1, 2]}
    with pytest.raises(pgsieve.PgsError):
        sieve.prp_gaps(503, 210, 5000, lists)  # row reaches past the distance array
    with pytest.raises(pgsieve.PgsError):
        sieve.prp_gaps(503, 4, 5000, {"m": [5], "start": [0], "n_prev": [0], "n_next": [0], "dist": []})
    res, _ = sieve.prp_gaps(503, 210, 5000, {"m": [], "start": [], "n_prev": [], "n_next": [], "dist": []})
    assert res == []
