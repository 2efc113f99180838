"""The drop-in combined_sieve CLI against the reference's own output
(tests/golden/cli.json, made by tests/golden/make_cli_goldens.py from the
reference built in oracle/_ref): set_defaults -- the d optimizer, the
automatic sieve length and max_prime (combined_sieve.cpp:160-344) -- and
main()'s validation (combined_sieve.cpp:86-135).  None of these cases sieves:
the CLI runs with no visible device, so the runs that would go on to sieve
(the automatic max_prime cases reach 1e11) stop with exit 1 at context
creation, and are compared on the lines printed before it."""
from __future__ import annotations

import json
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "prime-gap_gb300" / "_build" / "combined_sieve"
CASES = json.loads((ROOT / "tests" / "golden" / "cli.json").read_text())


def _auto(lines):
    return [l for l in lines if l.startswith(("AUTO SET", "WATCH"))]


@pytest.mark.parametrize("name", sorted(CASES))
def test_cli_matches_reference_before_sieving(built, tmp_path, name):
    case = CASES[name]
    (tmp_path / "unknowns").mkdir()
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")  # no device: nothing sieves
    p = subprocess.run(["stdbuf", "-oL", str(CLI), *case["args"].split()], cwd=tmp_path, env=env,
                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=120)
    out = p.stdout
    lines = out.splitlines()
    if case["compare"] == "all":
        assert lines == case["lines"]
        assert p.returncode == case["rc"]
    else:
        assert _auto(lines)[:len(case["lines"])] == case["lines"]
