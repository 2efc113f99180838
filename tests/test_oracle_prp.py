"""The probable-prime oracle against known answers and the reference's own
gap_test_simple runs (tests/golden/gaps.json, made by
tests/golden/make_gap_goldens.py from the reference built in oracle/_ref)."""
from __future__ import annotations

import hashlib
import json
import math
from pathlib import Path

import pytest

import pgo
import prp_oracle as po

GAPS = json.loads((Path(__file__).resolve().parent / "golden" / "gaps.json").read_text())

# base-2 strong pseudoprimes (OEIS A001262) pass; 561 and other Carmichael numbers fail
STRONG_PSP2 = [2047, 3277, 4033, 4681, 8321, 15841, 29341, 42799, 49141, 52633, 65281, 74665, 80581, 85489,
               88357]
MERSENNE_EXP = [5, 7, 13, 17, 19, 31, 61, 89, 107, 127, 521, 607, 1279]


def test_strong_prp2_small_numbers_against_trial_division():
    psp = set(STRONG_PSP2)
    for n in range(5, 90000, 2):
        is_prime = all(n % q for q in range(3, math.isqrt(n) + 1, 2))
        assert po.strong_prp2(n) == (is_prime or n in psp), n


def test_strong_prp2_large_known_numbers():
    for e in MERSENNE_EXP:
        assert po.strong_prp2((1 << e) - 1), e
        if e > 5:
            assert not po.strong_prp2((1 << e) + 1), e  # divisible by 3
    assert not po.strong_prp2(((1 << 127) - 1) * ((1 << 89) - 1))
    for c in (561, 1105, 1729, 2465, 2821, 6601, 8911):
        assert not po.strong_prp2(c), c


def test_k_log_matches_truncated_mantissa():
    k = po.primorial_k(907, 2190)
    assert k.bit_length() == 1240
    assert abs(po.k_log(k) - math.log(k)) < 1e-9
    # the mantissa is truncated, not rounded: K = 2^60 - 1 keeps 53 ones
    assert po.k_log((1 << 60) - 1) == math.log(((1 << 53) - 1) / (1 << 53)) + math.log(2) * 60


def _lists(g):
    text = pgo.method2(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"],
                       g["compression"], threads=8)
    assert hashlib.md5(text).hexdigest() == g["unknowns_md5"]
    return pgo.parse_unknowns(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"],
                              g["compression"], text)


def _subset(lists, rows):
    import numpy as np

    return {"m": lists["m"][rows], "start": lists["start"][rows], "n_prev": lists["n_prev"][rows],
            "n_next": lists["n_next"][rows], "dist": lists["dist"]} if len(rows) else lists


@pytest.mark.parametrize("name,rows", [
    ("fn1", [0, 1, 2, 3, 4, 5]),
    ("small_d7_odd", [0, 1, 2, 505, 923]),          # 505 and 923 run past SL
    ("overflow_503_210", [0, 10, 51, 57, 60, 61]),  # RLE file; 10-60 past SL
])
def test_gap_search_matches_reference_gap_test(name, rows):
    g = GAPS[name]
    lists = _subset(_lists(g), rows)
    k = po.primorial_k(g["p"], g["d"])
    got = po.gap_search(k, g["sieve_length"], lists)
    want = [g["gaps"][r] for r in rows]
    assert [[int(lists["m"][i]), r[0], r[1]] for i, r in enumerate(got)] == want
    for (prev_p, next_p, _, _, flags) in got:
        assert bool(flags & 1) == (prev_p > g["sieve_length"])
        assert bool(flags & 2) == (next_p > g["sieve_length"])


def test_gap_goldens_are_consistent():
    for name, g in GAPS.items():
        assert len(g["gaps"]) == pgo.plan(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"],
                                          g["max_prime"])["valid_ms"], name
        assert all(a > 0 and b > 0 for _, a, b in g["gaps"])
    assert GAPS["fn1"]["prp_tests"] == 2590
    assert GAPS["overflow_503_210"]["past_sieve_length"] > 100


def test_one_side_skip_rule():
    k = po.primorial_k(907, 2190)
    klog = po.k_log(k)
    # min_merit 18: skip when prev / (K_log + log m) < 7
    m = 17
    edge = 7 * (klog + math.log(m))
    assert po.skip_next_side(int(edge) - 1, m, klog, 18.0)
    assert not po.skip_next_side(int(edge) + 2, m, klog, 18.0)
    g = GAPS["fn1"]
    lists = _subset(_lists(g), [0, 1, 2])
    got = po.gap_search(k, g["sieve_length"], lists, min_merit=18.0, one_side_skip=True)
    for (prev_p, next_p, _, n_tests, flags), (m, want_prev, _) in zip(got, g["gaps"][:3]):
        assert prev_p == want_prev
        skipped = po.skip_next_side(prev_p, m, klog, 18.0)
        assert bool(flags & 4) == skipped and (next_p == 0) == skipped and (n_tests == 0) == skipped
