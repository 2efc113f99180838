"""The per-m path (pgs_method1, the reference's --method1: prime_gap_search,
combined_sieve.cpp:383-751) against the reference's files: each m's
large-prime marks come from its own bucket of surviving offsets, filled by
a counting pass and a filing pass of the large-prime phase, instead of the
atomic ORs of method2.  The reference checks its two methods against each
other (misc/tests.sh:62-67); here both are checked against its md5s."""
from __future__ import annotations

import hashlib
import json
import subprocess
from pathlib import Path

import pytest

import pgsieve

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "prime-gap_gb300" / "_build" / "combined_sieve"
MIX = Path(__file__).resolve().parent / "golden" / "mix_goldens.json"


def _spec(g) -> pgsieve.JobSpec:
    return pgsieve.JobSpec(g["p"], g["d"], g["mstart"], g["minc"], g["sieve_length"], g["max_prime"],
                           g.get("compression", 0))


@pytest.mark.parametrize("name", ["fn1", "fn1_rle", "fn1_bitcompressed", "fn2", "config1", "small_d1",
                                  "small_d7_odd", "small_d73_sl_odd", "small_d30030", "edge_maxprime_1M"])
def test_method1_matches_reference(sieve, goldens, name):
    g = goldens[name]
    assert hashlib.md5(sieve.method1(_spec(g))).hexdigest() == g["md5"], name


@pytest.mark.parametrize("name", ["config2", "config3"])
def test_method1_full_size(sieve, goldens, name):
    """Config 2 (2e9) and config 3 (1e10, 2.5e8 primes above 2^32, whose
    golden is the reference's own --method1 file)."""
    g = goldens[name]
    assert hashlib.md5(sieve.method1(_spec(g))).hexdigest() == g["md5"], name


def test_method1_64bit_mix_job(sieve):
    """A mix job past 2^32 (d = 210), against the reference's md5."""
    g = json.loads(MIX.read_text())["w64_503_210"]
    assert hashlib.md5(sieve.method1(_spec(g))).hexdigest() == g["md5"]


def test_cli_method1_file(built, goldens, tmp_path):
    """combined_sieve --method1 writes the .m1.txt file with the method2 bytes."""
    (tmp_path / "unknowns").mkdir()
    args = [str(CLI), "-p", "907", "-d", "2190", "--mstart", "1", "--minc", "200", "--max-prime", "100",
            "--sieve-length", "11000", "--save-unknowns", "--method1", "-qqq"]
    p = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    files = sorted(f.name for f in (tmp_path / "unknowns").iterdir())
    assert files == ["907_2190_1_200_s11000_l100M.m1.txt"], p.stdout
    data = (tmp_path / "unknowns" / files[0]).read_bytes()
    assert hashlib.md5(data).hexdigest() == goldens["fn1"]["md5"]


@pytest.mark.parametrize("form", [1, 6, 7])
def test_method1_other_large_forms(goldens, form):
    """The per-m path through the other large-prime kernel forms (warps alone
    with a walk list; K mod p inside the kernel), config 2 and a job past
    2^32, against the reference's md5s."""
    g64 = json.loads(MIX.read_text())["w64_503_210"]
    with pgsieve.Sieve(0, load_tuning=False) as s:
        for g in (goldens["config2"], g64):
            job = _spec(g)
            s.tuning_set(job, {"large_form": form})
            assert hashlib.md5(s.method1(job)).hexdigest() == g["md5"], form
