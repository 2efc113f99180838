"""The plain and batched paths against the reference's own files for the
seeded 64-job mix and for jobs whose primes cross 2^32.

tests/golden/mix_goldens.json holds the reference combined_sieve's md5 for
every job of workloads.mixed_jobs(64, seed=4) (P 503..3001, d in {1, 210,
2190, 30030}, minc 1e3..1e5, SL 5000..40000, max_prime 1e8..4e9) and for
eight jobs with max_prime 4.3e9..1.2e10 (64-bit K mod p, walk starts and
table windows), made by tests/golden/make_goldens.py --mix.
"""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import pytest

import pgsieve
import workloads

pytestmark = pytest.mark.gpu

MIX = json.loads((Path(__file__).resolve().parent / "golden" / "mix_goldens.json").read_text())
WIDE = sorted(k for k in MIX if k.startswith("w64_"))


def _spec(g) -> pgsieve.JobSpec:
    return pgsieve.JobSpec(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"],
                           g["compression"])


def test_mix_goldens_are_the_seeded_mix():
    jobs = workloads.mixed_jobs(64, seed=4)
    for i, j in enumerate(jobs):
        g = MIX[f"mix64_{i:02d}"]
        assert (g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"]) == (
            j.p, j.d, j.mstart, j.minc, j.sieve_length, j.max_prime)


def test_plain_mix64_matches_reference(sieve):
    bad = []
    for i in range(64):
        g = MIX[f"mix64_{i:02d}"]
        with sieve.method2_view(_spec(g)) as v:
            if hashlib.md5(v.view).hexdigest() != g["md5"] or len(v) != g["bytes"]:
                bad.append(i)
    assert not bad, [MIX[f"mix64_{i:02d}"] for i in bad]


def test_batch_mix64_matches_reference(sieve):
    """The whole 64-job mix in one graph-captured batch, replayed."""
    jobs = workloads.mixed_jobs(64, seed=4)
    with sieve.batch(jobs, lanes=8) as b:
        for _ in range(2):
            b.run(graph=True)
            bad = []
            for i in range(len(jobs)):
                with b.fetch_view(i) as v:
                    if hashlib.md5(v.view).hexdigest() != MIX[f"mix64_{i:02d}"]["md5"]:
                        bad.append(i)
            assert not bad, [str(jobs[i]) for i in bad]


def test_method2_batch_mix64_matches_reference(sieve):
    """pgs_method2_batch: host results for the whole mix in one call."""
    jobs = workloads.mixed_jobs(64, seed=4)
    views = sieve.method2_batch_views(jobs)
    try:
        got = [hashlib.md5(v.view).hexdigest() for v in views]
    finally:
        for v in views:
            v.close()
    want = [MIX[f"mix64_{i:02d}"]["md5"] for i in range(len(jobs))]
    assert got == want


@pytest.mark.parametrize("name", WIDE)
def test_plain_64bit_primes_match_reference(sieve, name):
    g = MIX[name]
    data = sieve.method2(_spec(g))
    assert hashlib.md5(data).hexdigest() == g["md5"]
    assert len(data) == g["bytes"]


def test_batch_64bit_primes_match_reference(sieve):
    """The jobs past 2^32 batched together (shared table windows above 2^32,
    K' mod p per P group)."""
    jobs = [_spec(MIX[n]) for n in WIDE]
    got = sieve.method2_batch(jobs)
    assert [hashlib.md5(x).hexdigest() for x in got] == [MIX[n]["md5"] for n in WIDE]
