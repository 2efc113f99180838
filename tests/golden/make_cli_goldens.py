"""Regenerate tests/golden/cli.json from the reference combined_sieve itself
(oracle/_ref/combined_sieve, built from the reference's sources by
oracle/build_ref.sh): its output and exit code for argument sets that stop
before or right after set_defaults (combined_sieve.cpp:74-135, 160-344) --
the d optimizer, the automatic sieve length and max_prime, and validation
failures.  Lines from set_defaults are kept; for the runs that go on to sieve
only those lines are compared.

    python tests/golden/make_cli_goldens.py
"""
from __future__ import annotations

import json
import subprocess
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
REF = ROOT / "oracle" / "_ref" / "combined_sieve"
OUT = Path(__file__).resolve().parent / "cli.json"

# (name, arguments, what to compare: "all" output lines or only "auto" lines)
CASES = [
    ("d_optimizer_907", "-p 907 -d 4 --mstart 1 --minc 100 --max-prime 100 --sieve-length 11000 --save-unknowns -qqq",
     "all"),
    ("d_optimizer_503_499", "-p 503 -d 1996 --mstart 1 --minc 100 --max-prime 100 --save-unknowns -qqq", "all"),
    ("auto_sl_1511_2190", "-p 1511 -d 2190 --mstart 1 --minc 1000 --max-prime 1 --save-unknowns -qqq", "auto"),
    ("auto_sl_907_210", "-p 907 -d 210 --mstart 100 --minc 5000 --max-prime 1 --save-unknowns -qqq", "auto"),
    ("auto_sl_503_1", "-p 503 -d 1 --mstart 1 --minc 300 --max-prime 1 --save-unknowns -qqq", "auto"),
    ("auto_sl_2003_30030", "-p 2003 -d 30030 --mstart 7 --minc 2000 --max-prime 1 --save-unknowns -qqq", "auto"),
    # goes on to sieve to 1e11: the reference is stopped after 20 s, its lines so far kept
    ("auto_max_prime_3001", "-p 3001 -d 2190 --mstart 1 --minc 10 --sieve-length 40000 --save-unknowns", "auto"),
    ("auto_max_prime_1511", "-p 1511 -d 2190 --mstart 1 --minc 10 --sieve-length 20000 --save-unknowns", "auto"),
    ("bad_sieve_length", "-p 907 -d 2190 --mstart 1 --minc 200 --max-prime 100 --sieve-length 100 --save-unknowns "
     "-qqq", "all"),
    ("no_save_unknowns", "-p 907 -d 2190 --mstart 1 --minc 200 --max-prime 100 --sieve-length 11000 -qqq", "all"),
]


def run(args: str, timeout: float = 20) -> tuple[int | None, str]:
    """Exit code (None when stopped at the timeout) and standard output."""
    with tempfile.TemporaryDirectory() as td:
        (Path(td) / "unknowns").mkdir()
        p = subprocess.Popen(["stdbuf", "-oL", str(REF), *args.split()], cwd=td, stdout=subprocess.PIPE,
                             stderr=subprocess.DEVNULL, text=True)
        try:
            out, _ = p.communicate(timeout=timeout)
            return p.returncode, out
        except subprocess.TimeoutExpired:
            p.kill()
            out, _ = p.communicate()
            return None, out


def auto_lines(text: str) -> list[str]:
    return [l for l in text.splitlines() if l.startswith(("AUTO SET", "WATCH"))]


def main():
    out = {}
    for name, args, what in CASES:
        rc, text = run(args)
        out[name] = {"args": args, "compare": what, "rc": rc,
                     "lines": text.splitlines() if what == "all" else auto_lines(text)}
        print(name, rc, len(out[name]["lines"]))
    OUT.write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
