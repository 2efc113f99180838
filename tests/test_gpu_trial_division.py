"""Trial-division spot checks of the GPU's output (the reference's
GMP_VALIDATE_FACTORS idea, combined_sieve.cpp:1017-1029, 1928-1933).

On config 2 (P=1511, primes to 2e9) and on a job whose primes run past
2^32, a seeded sample of surviving offsets must have no prime factor below
the sieve limit, and a seeded sample of offsets that the GPU removed (live
offsets: coprime to K, m*K + X odd) must have one.  The oracle finds the
smallest factor by trial division with its own K mod q over every prime up
to the limit.
"""
from __future__ import annotations

import json
import os
import random
from pathlib import Path

import pytest

import pgo
import pgsieve

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


def _small_primes(n):
    return [q for q in range(2, n + 1) if all(q % f for f in range(2, int(q ** 0.5) + 1))]


def _sample(job: dict, text: bytes, seed: int, rows: int = 8, per_row: int = 4):
    """(m, X, survives) triples from the file text."""
    rng = random.Random(seed)
    k_primes = [q for q in _small_primes(job["p"]) if job["d"] % q]
    k_odd = job["d"] % 2 == 0  # K = P#/d is odd when 2 | d
    lines = text.split(b"\n")[:-1]
    out = []
    for line in rng.sample(lines, min(rows, len(lines))):
        head, low, high = line.decode().split("|")
        m = int(head.split(":")[0])
        lows = [-int(v[1:]) for v in low.split()]
        highs = [int(v[1:]) for v in high.split()]
        surv = lows + highs
        for x in rng.sample(surv, min(per_row, len(surv))):
            out.append((m, x, True))
        keep = set(surv)
        removed = []
        for x in range(-job["sieve_length"], job["sieve_length"] + 1):
            if x == 0 or x in keep:
                continue
            if (m * (1 if k_odd else 0) + x) % 2 == 0:
                continue  # m*K + X even
            if any(x % q == 0 for q in k_primes):
                continue  # shares a factor with K: not live
            removed.append(x)
        for x in rng.sample(removed, min(per_row, len(removed))):
            out.append((m, x, False))
    return out


@pytest.mark.parametrize("which", ["config2", "w64_503_210"])
def test_trial_division_of_gpu_output(sieve, goldens, which):
    if which == "config2":
        g = goldens["config2"]
    else:
        g = json.loads((HERE / "golden" / "mix_goldens.json").read_text())[which]
    job = {k: g[k] for k in ("p", "d", "mstart", "minc", "sieve_length", "max_prime")}
    text = sieve.method2(pgsieve.JobSpec(**job))
    trip = _sample(job, text, seed=31 + job["p"])
    assert sum(1 for t in trip if t[2]) >= 16 and sum(1 for t in trip if not t[2]) >= 16
    f = pgo.trial_division(job, [t[0] for t in trip], [t[1] for t in trip], threads=os.cpu_count() or 8)
    limit = job["max_prime"]
    for (m, x, survives), factor in zip(trip, f):
        if survives:
            assert factor == 0, (m, x, factor)
        else:
            # a prime above P, or one of d's primes (they do not divide K)
            assert 0 < factor < limit and (factor > job["p"] or job["d"] % factor == 0), (m, x, factor)
