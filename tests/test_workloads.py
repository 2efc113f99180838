"""The seeded workloads are jobs the reference accepts, with the stated ranges."""
from __future__ import annotations

import pgsieve
import workloads


def test_mixed_jobs_valid_and_in_range(built):
    jobs = workloads.mixed_jobs(64, seed=4)
    assert len(jobs) == 64
    for j in jobs:
        assert pgsieve.plan(j)["rc"] == 0, j
        assert j.p in workloads.MIXED_P and j.d in workloads.MIXED_D
        assert 1 <= j.mstart < 10**8
        assert 1000 <= j.minc <= 100000
        assert 5000 <= j.sieve_length <= 40000 and j.sieve_length % 500 == 0
        assert 6 * j.p <= j.sieve_length <= 22 * j.p
        assert 10**8 <= j.max_prime <= 4 * 10**9 and j.max_prime % 10**6 == 0
    assert workloads.mixed_jobs(64, seed=4) == jobs  # seeded


def test_single_jobs_valid(built):
    for name in ("small", "large", "wide"):
        assert pgsieve.plan(workloads.single_job(name))["rc"] == 0


def test_poisson_arrivals():
    t = workloads.poisson_arrivals(1000, 50.0, seed=5)
    assert all(b > a for a, b in zip(t, t[1:]))
    assert 15 < t[-1] < 25
