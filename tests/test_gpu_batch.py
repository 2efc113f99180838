"""Batched and served method2 over the resident prime table.

Every job's unknowns file from the batched path (one CUDA graph over many
streams) and from the request server must be byte-identical to the same job
run alone on the plain path, which is itself pinned to the reference's
golden files and to the oracle.  The full 64-job mix and the jobs past 2^32
are checked against the reference's own md5s in test_gpu_mix_reference.py.
"""
from __future__ import annotations

import hashlib
import random
import threading
import time

import pytest

import pgo
import pgsieve
import workloads

pytestmark = pytest.mark.gpu


def _small_mix(n, seed, max_prime_cap=300_000_000):
    rng = random.Random(seed)
    jobs = []
    for _ in range(n):
        j = workloads.mixed_job(rng, compression=rng.choice([0, 0, 1, 2]))
        j.max_prime = min(j.max_prime, max_prime_cap)
        j.minc = min(j.minc, 5000)
        jobs.append(j)
    return jobs


def test_batch_goldens(sieve, goldens):
    names = ["fn1", "fn1_rle", "fn1_bitcompressed", "small_d30", "small_d7_odd", "small_d73_sl_odd",
             "edge_maxprime_1M", "ext_907_210"]
    jobs = [pgsieve.JobSpec(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"],
                            g["compression"]) for g in (goldens[n] for n in names)]
    with sieve.batch(jobs, lanes=4) as b:
        b.run(graph=False)
        for i, n in enumerate(names):
            assert hashlib.md5(b.fetch(i)).hexdigest() == goldens[n]["md5"], n


def test_batch_with_masks_in_global_memory(sieve, goldens):
    """A batch where one job's masks do not fit the tile kernel's shared
    memory (400,000 m of d = 105: the masks are read from global memory for
    every job of the launch) next to golden jobs: every output equals the
    same job alone on the plain path (itself checked against the oracle) or
    the reference's md5."""
    big = pgsieve.JobSpec(89, 105, 1000003, 400_000, 1000, 2_000_000, 1)
    names = ["fn1", "small_d7_odd", "config1"]
    jobs = [big] + [pgsieve.JobSpec(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"],
                                    g["compression"]) for g in (goldens[n] for n in names)]
    want_big = hashlib.md5(sieve.method2(big)).hexdigest()
    with sieve.batch(jobs, lanes=4) as b:
        for graph in (False, True):
            b.run(graph=graph)
            assert hashlib.md5(b.fetch(0)).hexdigest() == want_big, graph
            for i, n in enumerate(names, start=1):
                assert hashlib.md5(b.fetch(i)).hexdigest() == goldens[n]["md5"], (n, graph)


def test_batch_result_counts_match_plain(sieve):
    """Each batched job reports the rows, sieving primes and unknowns of the
    same job run alone (the bench's pairs come from these counts)."""
    jobs = _small_mix(8, 21) + [pgsieve.JobSpec(503, 210, 1234567, 300, 5000, 4_400_000_000)]
    want = []
    for j in jobs:
        st: dict = {}
        with sieve.prepare(j) as prep:
            prep.run(False)
            prep.fetch(st)
        want.append((st["rows"], st["primes"], st["unknowns"]))
    with sieve.batch(jobs, lanes=4) as b:
        b.run(graph=True)
        for i in range(len(jobs)):
            with b.fetch_view(i) as v:
                assert (v.res.rows, v.res.primes, v.res.unknowns) == want[i], jobs[i]
    for j, w in zip(jobs, want):
        assert pgsieve.plan(j)["valid_ms"] == w[0]


def test_batch_graph_replay_matches_plain(sieve):
    jobs = _small_mix(16, 11)
    want = [sieve.method2(j) for j in jobs]
    with sieve.batch(jobs, lanes=6) as b:
        for graph in (True, True, False):
            b.run(graph=graph)
            for i, j in enumerate(jobs):
                assert b.fetch(i) == want[i], (graph, j)


def test_batch_vs_oracle(sieve):
    jobs = _small_mix(6, 12, max_prime_cap=40_000_000)
    for j in jobs:
        j.minc = min(j.minc, 1500)
    got = sieve.method2_batch(jobs)
    for j, g in zip(jobs, got):
        want = pgo.method2(j.p, j.d, j.mstart, j.minc, j.sieve_length, j.max_prime, j.compression,
                           threads=16)
        assert g == want, j


def test_server_results_same_alone_and_in_mix(sieve):
    jobs = _small_mix(40, 13)
    want = [sieve.method2(j) for j in jobs]
    with sieve.server(hbm_budget=8 << 30, lanes=6) as srv:
        tickets = []
        for j in jobs:
            tickets.append(srv.submit(j))
            time.sleep(0.0005)
        outs = [srv.wait(t, timeout_ms=120_000) for t in tickets]
        st = srv.stats()
    for j, (data, lat), w in zip(jobs, outs, want):
        assert data == w, j
        assert lat > 0
    assert st["completed"] == len(jobs) and st["failed"] == 0
    assert st["max_inflight"] > 1  # requests overlapped on the device
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]


def test_server_budget_limits_inflight(sieve):
    """A budget below two jobs' footprint runs them one at a time."""
    jobs = _small_mix(6, 14)
    want = [sieve.method2(j) for j in jobs]
    with sieve.server(hbm_budget=1, lanes=4) as srv:
        tickets = [srv.submit(j) for j in jobs]
        outs = [srv.wait(t, timeout_ms=120_000)[0] for t in tickets]
        st = srv.stats()
    assert outs == want
    assert st["max_inflight"] == 1
    assert st["peak_bytes"] > 0


def test_server_concurrent_submitters(sieve):
    jobs = _small_mix(24, 15)
    want = {i: sieve.method2(j) for i, j in enumerate(jobs)}
    got = {}
    with sieve.server(hbm_budget=16 << 30, lanes=8) as srv:
        def client(ids):
            for i in ids:
                data, _ = srv.wait(srv.submit(jobs[i]), timeout_ms=120_000)
                got[i] = data

        threads = [threading.Thread(target=client, args=(range(k, len(jobs), 4),)) for k in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    assert got == want


def test_server_kmod_cache_reuse(sieve):
    """Requests with the same (P, d) reuse K mod p; results stay identical,
    also when the cache budget forces evictions."""
    rng = random.Random(17)
    base = workloads.mixed_job(rng)
    jobs = []
    for k in range(6):
        j = workloads.mixed_job(rng, compression=k % 3)
        j.p, j.d = base.p, base.d
        j.sieve_length = base.sieve_length
        j.max_prime = min(j.max_prime, 600_000_000)
        j.minc = min(j.minc, 4000)
        jobs.append(j)
    want = [sieve.method2(j) for j in jobs]
    for budget in (64 << 30, 1):
        with sieve.server(hbm_budget=budget, lanes=3) as srv:
            outs = []
            for j in jobs:  # one at a time: each later request finds the entry
                outs.append(srv.wait(srv.submit(j), timeout_ms=120_000)[0])
            st = srv.stats()
        assert outs == want
        assert st["kmod_fills"] >= 1
        if budget > 1:
            assert st["kmod_hits"] >= len(jobs) - 1


def test_server_rejects_bad_job_without_stalling(sieve):
    good = _small_mix(2, 16)
    bad = pgsieve.JobSpec(503, 210, 1, 100, 100, 10_000_000)  # SL < 6P
    with sieve.server(hbm_budget=8 << 30, lanes=2) as srv:
        t0 = srv.submit(good[0])
        tb = srv.submit(bad)
        t1 = srv.submit(good[1])
        with pytest.raises(pgsieve.PgsError) as ei:
            srv.wait(tb, timeout_ms=60_000)
        assert ei.value.code == pgsieve.PGS_EINVAL
        assert srv.wait(t0, timeout_ms=60_000)[0] == sieve.method2(good[0])
        assert srv.wait(t1, timeout_ms=60_000)[0] == sieve.method2(good[1])
