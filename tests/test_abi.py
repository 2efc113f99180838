"""libpgsieve's C ABI on the CPU: every declared symbol is exported, host-side
job planning matches the reference's derived parameters, and invalid jobs are
rejected with the reference's validation rules.  No kernel runs here."""
from __future__ import annotations

import ctypes
import subprocess

import pytest

import pgo
import pgsieve

SYMBOLS = [
    "pgs_create", "pgs_destroy", "pgs_last_error", "pgs_set_stream", "pgs_get_stream",
    "pgs_method2", "pgs_result_free", "pgs_prepare", "pgs_run", "pgs_fetch", "pgs_prepared_free",
    "pgs_plan_job", "pgs_stage_ms", "pgs_int_peak", "pgs_primes", "pgs_k_mod_p", "pgs_modulo_search", "pgs_large_hits",
    "pgs_version", "pgs_table_reserve", "pgs_batch_prepare", "pgs_batch_run", "pgs_batch_fetch",
    "pgs_batch_free", "pgs_method2_batch", "pgs_server_start", "pgs_server_submit", "pgs_server_wait",
    "pgs_server_stats_get", "pgs_server_stop", "pgs_large_hits_static", "pgs_fetch_unknowns",
    "pgs_parse_unknowns", "pgs_unknowns_free", "pgs_prp_test", "pgs_prp_gaps", "pgs_prp_gaps_prepared",
]


def test_header_declares_expected_symbols():
    assert set(SYMBOLS) <= set(pgsieve.header_symbols())


def test_library_exports_every_header_symbol(built):
    lib = ctypes.CDLL(str(pgsieve.LIB_PATH))
    for name in pgsieve.header_symbols():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(pgsieve.LIB_PATH)], capture_output=True,
                         text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    assert set(pgsieve.header_symbols()) <= exported


def test_version(built):
    assert b"sm_103a" in pgsieve.load().pgs_version()


JOBS = [
    (907, 2190, 1, 200, 11000, 100_000_000),
    (953, 1, 1, 10000, 8000, 20_000_000),
    (503, 210, 1234567, 10000, 5000, 100_000_000),
    (1511, 2190, 12345679, 100000, 20000, 2_000_000_000),
    (3001, 2190, 123457, 100000, 40000, 10_000_000_000),
    (797, 30030, 123, 20000, 9000, 150_000_000),
    (557, 73, 1000003, 1500, 4001, 40_000_000),
]


@pytest.mark.parametrize("job", JOBS)
def test_plan_matches_oracle(built, job):
    p, d, ms, mi, sl, mp = job
    got = pgsieve.plan(pgsieve.JobSpec(p, d, ms, mi, sl, mp))
    want = pgo.plan(p, d, ms, mi, sl, mp)
    assert got["rc"] == 0 and want["rc"] == 0
    for k in ("valid_ms", "coprime_x", "small_threshold", "medium_threshold"):
        assert got[k] == want[k], k
    # same prime set: the library sieves up to a bound, the oracle reports the last prime
    import sympy

    assert want["prime_limit"] <= got["prime_limit"] < sympy.nextprime(want["prime_limit"])
    assert got["filename"] == "unknowns/" + pgsieve.JobSpec(p, d, ms, mi, sl, mp).filename


@pytest.mark.parametrize("job,rc", [
    ((907, 2190, 0, 200, 11000, 100_000_000), pgsieve.PGS_EINVAL),       # mstart = 0
    ((907, 2190, 1, 0, 11000, 100_000_000), pgsieve.PGS_EINVAL),         # minc = 0
    ((908, 2190, 1, 200, 11000, 100_000_000), pgsieve.PGS_EINVAL),       # p not prime
    ((907, 2190, 1, 200, 3000, 100_000_000), pgsieve.PGS_EINVAL),        # SL < 6P
    ((907, 2190, 1, 200, 30000, 100_000_000), pgsieve.PGS_EINVAL),       # SL > 22P
    ((907, 2190, 1, 200, 11001, 100_000_000), pgsieve.PGS_EINVAL),       # SL not coprime (3 | 11001)
    ((907, 2190, 10**10, 2, 11000, 100_000_000), pgsieve.PGS_EINVAL),    # mstart + minc > 1e10+1
    ((907, 2190, 1, 200, 11000, 50_000_000_000_000), pgsieve.PGS_EINVAL),  # > 40 trillion
    ((907, 1822, 1, 200, 11000, 100_000_000), pgsieve.PGS_EABORT),       # d = 2*911 does not divide P#
])
def test_plan_rejects_like_reference(built, job, rc):
    assert pgsieve.plan(pgsieve.JobSpec(*job))["rc"] == rc


def test_create_without_gpu_fails_cleanly(built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert pgsieve.load().pgs_create(0, ctypes.byref(h)) == pgsieve.PGS_ENODEV
    with pytest.raises(pgsieve.PgsError):
        pgsieve.Sieve(0)


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(FileNotFoundError):
        pgsieve.load(tmp_path / "nope.so")
