"""ORACLE -- test infrastructure only.

Pure-Python restatement (big integers) of the reference's probable-prime gap
search over unknown lists, the checker of the device PRP path.  Only tests,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it.  Pinned
against the reference's own gap_test_simple runs (tests/golden/gaps.json).

* strong_prp2: the reference's GPU Miller-Rabin with one base, 2
  (miller_rabin.h:211-245 with ROUNDS = 1, gap_test_gpu.cu:81).  Its squaring
  loop runs up to s times for N - 1 = d 2^s (one more than the textbook s - 1);
  restated as is.  The extra squaring never changes a verdict: 2^(N-1) = -1
  mod N has no odd solution N > 1, since the order of 2 modulo each prime p
  dividing N would need 2-adic valuation v2(N-1) + 1 <= v2(p - 1), making
  N = 1 mod 2^(v2(N-1)+1).
* gap_search: nearest-first tests of each side's unknowns
  (gap_test_common.cpp:139-158, gap_test_gpu.cu:431-470), past the sieve
  length the first probable prime beyond SL (mpz_prevprime / mpz_nextprime,
  gap_test_common.cpp:160-178, gap_test_gpu.cu:258-285), and gap_test_gpu's
  one-side skip (gap_test_gpu.cu:570-596).
"""
from __future__ import annotations

import math
import struct


def strong_prp2(n: int) -> bool:
    """Base-2 strong probable-prime test with the reference's loop bound."""
    if n < 5 or n % 2 == 0:
        raise ValueError("odd n >= 5 expected")
    d = n - 1
    s = (d & -d).bit_length() - 1
    d >>= s
    x = pow(2, d, n)
    if x == 1 or x == n - 1:
        return True
    if s == 1:
        return False
    count = s
    while True:
        x = x * x % n
        if x == n - 1:
            return True
        count -= 1
        if count == 0 or x == 1:
            return False


def primorial_k(p: int, d: int) -> int:
    """K = p# / d (gap_common.cpp:116-121)."""
    k = 1
    for q in range(2, p + 1):
        if all(q % r for r in range(2, int(q ** 0.5) + 1)):
            k *= q
    if k % d:
        raise ValueError("d does not divide p#")
    return k // d


def k_log(k: int) -> float:
    """_log(K) = log(mantissa) + log(2) * exp with GMP's truncated 53-bit
    mantissa in [0.5, 1) (gap_common.cpp:100-104)."""
    b = k.bit_length()
    top = k >> (b - 53) if b > 53 else k << (53 - b)
    return math.log(top / float(1 << 53)) + math.log(2) * b


def _f32(x: float) -> float:
    return struct.unpack("f", struct.pack("f", x))[0]


def skip_next_side(prev_p: int, m: int, klog: float, min_merit: float) -> bool:
    """gap_test_gpu.cu:577-590: float prev_merit = prev_p / (K_log + log(m));
    skip when prev_merit < min_merit / 2 - 2 (float arithmetic)."""
    mm = _f32(min_merit)
    threshold = _f32(_f32(mm / 2) - 2)
    return _f32(prev_p / (klog + math.log(m))) < threshold


def _past_sieve(center: int, sl: int, sign: int) -> int:
    x = sl + 1
    while True:
        n = center + sign * x
        if n % 2 and strong_prp2(n):
            return x
        x += 1


def gap_search(k: int, sl: int, lists: dict, min_merit: float = 18.0, one_side_skip: bool = False):
    """Per row of lists (m, n_prev, n_next, start, dist as from parse_unknowns):
    (prev_p, next_p, p_tests, n_tests, flags) with flags bit 0 = prev past SL,
    bit 1 = next past SL, bit 2 = next side skipped."""
    klog = k_log(k)
    out = []
    for i in range(len(lists["m"])):
        m = int(lists["m"][i])
        a = int(lists["start"][i])
        n_prev, n_next = int(lists["n_prev"][i]), int(lists["n_next"][i])
        prev = [int(x) for x in lists["dist"][a:a + n_prev]]
        nxt = [int(x) for x in lists["dist"][a + n_prev:a + n_prev + n_next]]
        center = m * k
        flags = 0
        prev_p = next_p = p_tests = n_tests = 0
        for j, x in enumerate(prev):
            if strong_prp2(center - x):
                prev_p, p_tests = x, j + 1
                break
        else:
            prev_p, p_tests, flags = _past_sieve(center, sl, -1), len(prev), flags | 1
        if one_side_skip and skip_next_side(prev_p, m, klog, min_merit):
            out.append((prev_p, 0, p_tests, 0, flags | 4))
            continue
        for j, x in enumerate(nxt):
            if strong_prp2(center + x):
                next_p, n_tests = x, j + 1
                break
        else:
            next_p, n_tests, flags = _past_sieve(center, sl, 1), len(nxt), flags | 2
        out.append((prev_p, next_p, p_tests, n_tests, flags))
    return out
