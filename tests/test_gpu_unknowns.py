"""Unknown lists for gap_stats: read off the device, or parsed on the device.

Every route -- the lists a sieved job leaves on the device, and the device
parse of an unknowns file in each of the three formats -- must give exactly
the lists of the oracle's restatement of parse_unknown_line
(gap_common.cpp:1186-1360), which is itself checked against the unknowns read
straight off the oracle's sieve (test_oracle_lists.py).
"""
from __future__ import annotations

import numpy as np
import pytest

import pgo
import pgsieve

pytestmark = pytest.mark.gpu

JOBS = [
    (907, 2190, 1, 200, 11000, 100_000_000),        # FN1 (misc/tests.sh)
    (503, 210, 1234567, 3000, 5000, 100_000_000),
    (557, 73, 1000003, 1500, 4001, 40_000_000),      # d odd, SL odd
    (521, 7, 999, 500, 7000, 10_000_000),
    (509, 1, 77, 300, 5000, 3_000_000),
    (1009, 30030, 98765, 2000, 9500, 300_000_000),
]


def _same(a: dict, b: dict):
    for k in ("m", "n_prev", "n_next", "start", "dist"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("job", JOBS)
@pytest.mark.parametrize("comp", [0, 1, 2])
def test_all_routes_match_oracle(sieve, job, comp):
    want = pgo.method2_lists(*job, threads=16)
    spec = pgsieve.JobSpec(*job, comp)
    text = sieve.method2(spec)
    _same(pgo.parse_unknowns(*job, comp, text), want)  # the same bytes as the oracle's file
    _same(sieve.parse_unknowns(spec, text), want)
    with sieve.prepare(spec) as prep:
        prep.run(False)
        _same(prep.unknowns(), want)


def test_config2_formats_agree(sieve, goldens):
    """Full size (P=1511, d=2190, minc=1e5, SL=2e4, max_prime=2e9): the three
    formats decode to the device lists, whose counts match the text headers."""
    g = goldens["config2"]
    base = (g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"])
    spec0 = pgsieve.JobSpec(*base, 0)
    with sieve.prepare(spec0) as prep:
        prep.run(False)
        direct = prep.unknowns()
        text0 = prep.fetch()
    assert len(direct["m"]) == 26301
    _same(sieve.parse_unknowns(spec0, text0), direct)
    for comp in (1, 2):
        spec = pgsieve.JobSpec(*base, comp)
        _same(sieve.parse_unknowns(spec, sieve.method2(spec)), direct)
    lines = text0.split(b"\n")[:-1]
    heads = [ln.split(b" ", 4) for ln in lines[:50]]
    assert [int(h[0]) for h in heads] == list(direct["m"][:50])
    assert [-int(h[2]) for h in heads] == list(direct["n_prev"][:50])
    assert [int(h[3]) for h in heads] == list(direct["n_next"][:50])


def test_parse_rejects_bad_files(sieve):
    job = JOBS[0]
    spec = pgsieve.JobSpec(*job, 0)
    text = sieve.method2(spec)
    with pytest.raises(pgsieve.PgsError) as e:
        sieve.parse_unknowns(spec, text[: len(text) // 2])  # rows missing
    assert e.value.code == pgsieve.PGS_EINVAL
    with pytest.raises(pgsieve.PgsError):
        sieve.parse_unknowns(pgsieve.JobSpec(*job, 2), text)  # plain text, bitcompressed job
    with pytest.raises(pgsieve.PgsError):
        sieve.parse_unknowns(spec, text.replace(b" | ", b" # ", 1))
