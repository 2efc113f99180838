"""The oracle's restatement of parse_unknown_line (gap_common.cpp:1186-1360).

Parsing an unknowns file of any compression must give the same per-m lists
as reading them straight off the sieve; the text itself is pinned to the
reference's goldens (test_oracle_golden.py).  Malformed lines are rejected
where the reference asserts.
"""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

import pgo

JOBS = [
    (907, 2190, 1, 200, 11000, 100_000_000),        # FN1 (misc/tests.sh)
    (503, 210, 1234567, 3000, 5000, 100_000_000),
    (557, 73, 1000003, 1500, 4001, 40_000_000),      # d odd, SL odd
    (521, 7, 999, 500, 7000, 10_000_000),
    (509, 1, 77, 300, 5000, 3_000_000),
]


@pytest.mark.parametrize("job", JOBS)
@pytest.mark.parametrize("comp", [0, 1, 2])
def test_parse_matches_direct_lists(built, job, comp):
    direct = pgo.method2_lists(*job, threads=8)
    text = pgo.method2(*job, comp, threads=8)
    parsed = pgo.parse_unknowns(*job, comp, text)
    for k in direct:
        assert np.array_equal(direct[k], parsed[k]), k
    assert int(direct["n_prev"].sum() + direct["n_next"].sum()) == len(direct["dist"])


def test_fn1_text_is_the_golden(built, goldens):
    text = pgo.method2(907, 2190, 1, 200, 11000, 100_000_000, 0, threads=8)
    assert hashlib.md5(text).hexdigest() == goldens["fn1"]["md5"]


def test_parse_rejects_malformed(built):
    job = (907, 2190, 1, 200, 11000, 100_000_000)
    text = pgo.method2(*job, 2, threads=8)
    first, rest = text.split(b"\n", 1)
    m, colon, total, nbytes, bars, raw = first.split(b" ", 5)
    bad = b" ".join([m, colon, total, str(int(nbytes) + 1).encode(), bars, raw]) + b"\n" + rest
    with pytest.raises(RuntimeError):
        pgo.parse_unknowns(*job, 2, bad)
    with pytest.raises(RuntimeError):
        pgo.parse_unknowns(*job, 0, text.split(b"\n", 1)[1])  # a row short
