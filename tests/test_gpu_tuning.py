"""Tuned knobs change the time, never the bytes: plain and one-call outputs
with extreme knob settings against the reference's golden md5s (batched jobs
keep the default knobs and must match too), and pgs_tune's result stored for
the job's class."""
from __future__ import annotations

import hashlib

import pytest

import pgsieve

pytestmark = pytest.mark.gpu

EXTREMES = [
    {"direct_steps": 8, "item_steps": 32, "heavy_steps": 1024, "rows_per_cta": 4, "text_chunks": 1,
     "kmod_lsb_limbs": 8, "large_form": 1},
    {"direct_steps": 48, "item_steps": 128, "heavy_steps": 16384, "rows_per_cta": 32, "text_chunks": 2,
     "kmod_lsb_limbs": 1 << 20, "large_form": 0},
    {"direct_steps": 1, "item_steps": 64, "heavy_steps": 256, "rows_per_cta": 1, "text_chunks": 3,
     "kmod_lsb_limbs": 1, "large_form": 1},
    # K mod p inside the large-prime kernel: most significant limb first, pooled
    {"direct_steps": 24, "item_steps": 32, "heavy_steps": 2048, "rows_per_cta": 8, "text_chunks": 4,
     "kmod_lsb_limbs": 1 << 20, "large_form": 6},
    # least significant limb first, warps alone
    {"direct_steps": 16, "item_steps": 64, "heavy_steps": 4096, "rows_per_cta": 16, "text_chunks": 1,
     "kmod_lsb_limbs": 1, "large_form": 7},
]
NAMES = ["fn1", "fn1_bitcompressed", "small_d7_odd", "small_d30030", "config1", "edge_maxprime_1M"]


def _spec(g) -> pgsieve.JobSpec:
    return pgsieve.JobSpec(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"],
                           g["compression"])


@pytest.mark.parametrize("knobs", EXTREMES)
def test_knobs_keep_bytes_plain_and_batched(goldens, knobs):
    with pgsieve.Sieve(0, load_tuning=False) as s:
        jobs = [_spec(goldens[n]) for n in NAMES]
        for j in jobs:
            s.tuning_set(j, knobs)
            assert s.tuning_get(j) == (knobs, True)
        for n, j in zip(NAMES, jobs):
            assert hashlib.md5(s.method2(j)).hexdigest() == goldens[n]["md5"], (n, knobs)
            with s.prepare(j) as prep:
                prep.run(False)
                assert hashlib.md5(prep.fetch()).hexdigest() == goldens[n]["md5"], (n, knobs)
        got = s.method2_batch(jobs)
        assert [hashlib.md5(x).hexdigest() for x in got] == [goldens[n]["md5"] for n in NAMES]


def test_tune_stores_class_result(goldens, tmp_path):
    with pgsieve.Sieve(0, load_tuning=False) as s:
        job = _spec(goldens["config1"])
        knobs, ms_def, ms_tuned = s.tune(job, reps=2)
        assert ms_def > 0 and ms_tuned > 0
        assert s.tuning_get(job) == (knobs, True)
        f = tmp_path / "t.tsv"
        assert s.tuning_save(f) == 1
        assert hashlib.md5(s.method2(job)).hexdigest() == goldens["config1"]["md5"]
    with pgsieve.Sieve(0, load_tuning=False) as s2:
        assert s2.tuning_get(job)[1] is False
        assert s2.tuning_load(f) == 1
        assert s2.tuning_get(job) == (knobs, True)


@pytest.mark.parametrize("form", [1, 2, 5, 6, 7])
@pytest.mark.parametrize("name", ["config2", "w64_503_210"])
def test_large_forms_full_size(goldens, name, form):
    """The other large-prime forms -- warps alone with a walk list (bit 0), K
    mod p inside the large-prime kernel for 32-bit (bit 1) and 64-bit primes
    (bit 2) -- on config 2 and on a job past 2^32, against the reference's
    md5."""
    import json
    from pathlib import Path

    g = goldens.get(name) or json.loads(
        (Path(__file__).resolve().parent / "golden" / "mix_goldens.json").read_text())[name]
    with pgsieve.Sieve(0, load_tuning=False) as s:
        job = _spec(g)
        s.tuning_set(job, {"large_form": form})
        assert hashlib.md5(s.method2(job)).hexdigest() == g["md5"]


def test_fused_kmod_config3(goldens):
    """K mod p of 64-bit primes inside the large-prime kernel, config 3 at
    full size (2.5e8 primes above 2^32), against the reference's md5."""
    with pgsieve.Sieve(0, load_tuning=False) as s:
        job = _spec(goldens["config3"])
        s.tuning_set(job, {"large_form": 6})
        assert hashlib.md5(s.method2(job)).hexdigest() == goldens["config3"]["md5"]
