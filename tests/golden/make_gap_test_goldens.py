"""Regenerate tests/golden/gap_test_logs.json from the reference itself: the
output of the reference's gap_test_simple (oracle/_ref/gap_test_simple, built
from the reference's sources by oracle/build_ref.sh) on unknowns files that
the reference combined_sieve writes, with the timing fields masked as the
reference's own test script does (misc/tests.sh:118-119).

    python tests/golden/make_gap_test_goldens.py
"""
from __future__ import annotations

import json
import re
import shutil
import subprocess
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
SIEVE = ROOT / "oracle" / "_ref" / "combined_sieve"
GAP_TEST = ROOT / "oracle" / "_ref" / "gap_test_simple"
OUT = Path(__file__).resolve().parent / "gap_test_logs.json"

# (name, sieve arguments, unknowns file, gap_test arguments after -u <file>)
CASES = [
    ("fn1_tests_sh", "-p 907 -d 2190 --mstart 1 --minc 200 --max-prime 100 --sieve-length 11000",
     "907_2190_1_200_s11000_l100M.m1.txt", "--min-merit 8 -q"),
    ("fn1_all", "-p 907 -d 2190 --mstart 1 --minc 200 --max-prime 100 --sieve-length 11000",
     "907_2190_1_200_s11000_l100M.txt", "--min-merit 0 -q"),
    ("d7_odd_past_sl", "-p 509 -d 7 --mstart 31337 --minc 2000 --max-prime 10 --sieve-length 3500",
     "509_7_31337_2000_s3500_l10M.txt", "--min-merit 10 -q"),
    ("rle_mskip", "-p 503 -d 210 --mstart 1234567 --minc 20000 --max-prime 10 --sieve-length 3024 --rle",
     "503_210_1234567_20000_s3024_l10M.txt", "--min-merit 6 --mskip 1244567 -q"),
    ("bitcompressed_quiet", "-p 521 -d 30 --mstart 2024 --minc 1500 --max-prime 40 --sieve-length 5000 "
     "--bitcompressed", "521_30_2024_1500_s5000_l40M.txt", "--min-merit 5 -q -q"),
]


def mask(text: str) -> list[str]:
    """misc/tests.sh:118-119: rates to XX.YY, elapsed seconds to Z."""
    text = re.sub(r"[0-9.]+( ?)(tests)?/sec\)", r"XX.YY\1\2/sec)", text)
    text = re.sub(r"[0-9]+ sec", "Z sec", text)
    return text.splitlines()


def main():
    out = {}
    for name, sieve_args, fn, args in CASES:
        with tempfile.TemporaryDirectory() as td:
            tdp = Path(td)
            (tdp / "unknowns").mkdir()
            subprocess.run([str(SIEVE), "-qqq", "--save-unknowns", "-t", "1", *sieve_args.split()], cwd=tdp,
                           capture_output=True)  # exits 1 after saving without a search database
            made = list((tdp / "unknowns").iterdir())
            assert len(made) == 1, made
            if made[0].name != fn:
                shutil.copy(made[0], tdp / "unknowns" / fn)
            p = subprocess.run(["stdbuf", "-oL", str(GAP_TEST), "-u", fn, *args.split()], cwd=tdp,
                               capture_output=True, text=True, timeout=600)
        out[name] = {"sieve_args": sieve_args, "unknowns_file": fn, "args": args, "rc": p.returncode,
                     "lines": mask(p.stdout)}
        print(name, p.returncode, len(out[name]["lines"]))
    OUT.write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
