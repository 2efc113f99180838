"""Seeded synthetic method2 workloads: the single-job sizes, the 64-job mixed
batch and the served request stream.

Job parameters obey the reference's own argument rules so every job is one
the reference CLI accepts: sieve_length in [6P, 22P] (combined_sieve.cpp:97-103),
kept a multiple of 500 so the coprimality rule of combined_sieve.cpp:86-95 does
not apply, d | P#, and max_prime a whole number of millions (--max-prime is
given in millions, gap_common.cpp:936-938).
"""
from __future__ import annotations

import math
import random

from pgsieve import JobSpec

MIXED_P = (503, 797, 1009, 1511, 2003, 3001)
MIXED_D = (1, 210, 2190, 30030)


def single_job(name: str, seed: int = 0) -> JobSpec:
    """The three single-job sizes (m_start drawn from the seed)."""
    rng = random.Random(seed)
    if name == "small":  # P=503, d=210, minc=1e4, SL=5000, max_prime=1e8
        return JobSpec(503, 210, rng.randrange(10**5, 10**7), 10000, 5000, 100_000_000)
    if name == "large":  # P=1511, d=2190, minc=1e5, SL=2e4, max_prime=2e9
        return JobSpec(1511, 2190, rng.randrange(10**6, 10**8), 100000, 20000, 2_000_000_000)
    if name == "wide":  # P=3001, d=2190, minc=1e5, SL=4e4, max_prime=1e10
        return JobSpec(3001, 2190, rng.randrange(1, 10**6), 100000, 40000, 10_000_000_000)
    raise ValueError(name)


def _log_uniform(rng: random.Random, lo: float, hi: float) -> float:
    return math.exp(rng.uniform(math.log(lo), math.log(hi)))


def mixed_job(rng: random.Random, compression: int = 0) -> JobSpec:
    """One job of the heterogeneous mix: P, d, m_start, m_inc (log-uniform
    1e3..1e5), SL (5000..40000 within the reference's [6P, 22P]) and
    max_prime (log-uniform 1e8..4e9)."""
    P = rng.choice(MIXED_P)
    d = rng.choice(MIXED_D)
    mstart = rng.randrange(1, 10**8)
    minc = int(round(_log_uniform(rng, 1e3, 1e5)))
    lo = max(5000, 6 * P)
    hi = min(40000, 22 * P)
    sl = rng.randrange((lo + 499) // 500, hi // 500 + 1) * 500
    max_prime = int(round(_log_uniform(rng, 1e8, 4e9) / 1e6)) * 1_000_000
    return JobSpec(P, d, mstart, minc, sl, max_prime, compression)


def mixed_jobs(n: int = 64, seed: int = 4) -> list[JobSpec]:
    rng = random.Random(seed)
    return [mixed_job(rng) for _ in range(n)]


def poisson_arrivals(n: int, rate_per_s: float, seed: int = 5) -> list[float]:
    """Arrival times (s from start) of n requests at the given mean rate."""
    rng = random.Random(seed)
    t, out = 0.0, []
    for _ in range(n):
        t += rng.expovariate(rate_per_s)
        out.append(t)
    return out


def main(argv: list[str] | None = None) -> int:
    """python prime-gap_gb300/workloads.py batch64 [--lanes N] [--graph]: one
    batched run of the 64-job mix over the resident table (a short command to
    profile the batched path alone); prints the device time."""
    import argparse

    import pgsieve

    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["batch64"])
    ap.add_argument("--lanes", type=int, default=8)
    ap.add_argument("--graph", action="store_true")
    a = ap.parse_args(argv)
    s = pgsieve.Sieve(0)
    try:
        s.reserve_table(4_000_000_000)
        with s.batch(mixed_jobs(64, seed=4), lanes=a.lanes) as b:
            print(f"batch64: {b.run(graph=a.graph):.2f} ms")
    finally:
        s.close()
    return 0


if __name__ == "__main__":
    import sys

    sys.exit(main())
