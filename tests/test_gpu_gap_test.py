"""The drop-in gap_test CLI against the reference's gap_test_simple output
(tests/golden/gap_test_logs.json, made by tests/golden/make_gap_test_goldens.py
from the reference built in oracle/_ref): the unknowns files come from the
device sieve, the parse and the probable-prime search run on the device, and
the printed gaps and stats lines must match the reference's, timing fields
masked as misc/tests.sh:118-119 masks them."""
from __future__ import annotations

import json
import re
import subprocess
from pathlib import Path

import pytest

import pgsieve

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
GAP_TEST = ROOT / "prime-gap_gb300" / "_build" / "gap_test"
CASES = json.loads((ROOT / "tests" / "golden" / "gap_test_logs.json").read_text())


def _mask(text: str) -> list[str]:
    text = re.sub(r"[0-9.]+( ?)(tests)?/sec\)", r"XX.YY\1\2/sec)", text)
    text = re.sub(r"[0-9]+ sec", "Z sec", text)
    return text.splitlines()


def _spec(sieve_args: str) -> pgsieve.JobSpec:
    a = sieve_args.split()
    val = {a[i]: a[i + 1] for i in range(len(a) - 1) if a[i].startswith("-") and not a[i + 1].startswith("-")}
    comp = 1 if "--rle" in a else 2 if "--bitcompressed" in a else 0
    return pgsieve.JobSpec(int(val["-p"]), int(val["-d"]), int(val["--mstart"]), int(val["--minc"]),
                           int(val["--sieve-length"]), int(val["--max-prime"]) * 1_000_000, comp)


@pytest.mark.parametrize("name", sorted(CASES))
def test_gap_test_cli_matches_reference(built, sieve, tmp_path, name):
    case = CASES[name]
    (tmp_path / "unknowns").mkdir()
    (tmp_path / "unknowns" / case["unknowns_file"]).write_bytes(sieve.method2(_spec(case["sieve_args"])))
    p = subprocess.run([str(GAP_TEST), "-u", case["unknowns_file"], *case["args"].split()], cwd=tmp_path,
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == case["rc"], p.stdout[-2000:]
    assert _mask(p.stdout) == case["lines"]


def test_gap_test_cli_one_side_skip(built, sieve, tmp_path):
    """gap_test_gpu's skip: the next side is searched only after a previous
    gap of merit at least min_merit/2 - 2; the gaps printed are a subset of
    the full run's."""
    case = CASES["fn1_all"]
    (tmp_path / "unknowns").mkdir()
    (tmp_path / "unknowns" / case["unknowns_file"]).write_bytes(sieve.method2(_spec(case["sieve_args"])))
    run = lambda *extra: subprocess.run([str(GAP_TEST), "-u", case["unknowns_file"], "--min-merit", "8", "-q",
                                         *extra], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    full, skip = run(), run("--one-side-skip")
    assert full.returncode == 0 and skip.returncode == 0
    gaps = lambda out: [l for l in out.splitlines() if re.match(r"^\d+ +\d+\.\d+ ", l)]
    assert set(gaps(skip.stdout)) <= set(gaps(full.stdout))
    assert len(gaps(skip.stdout)) >= 1
