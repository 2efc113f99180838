"""Regenerate tests/golden/gaps.json from the reference itself.

For each job, the reference combined_sieve (oracle/_ref/combined_sieve, built
from the reference's sources by oracle/build_ref.sh) writes the unknowns file,
and the reference gap_test_simple (oracle/_ref/gap_test_simple, same build)
runs on it with --min-merit 0, so that it prints one gap line per valid m:
"gap merit  m * P#/d -prev to +next" (gap_test_simple.cpp:185-190).  Its
primality test is GMP's mpz_probab_prime_p(N, 25) over the unknowns, nearest
first on each side, and mpz_prevprime / mpz_nextprime past the sieve length
(gap_test_common.cpp:128-181).  Recorded per job: the unknowns file's md5,
every (m, prev, next) and the total PRP tests of the last stats line.

    python tests/golden/make_gap_goldens.py
"""
from __future__ import annotations

import hashlib
import json
import re
import subprocess
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
SIEVE = ROOT / "oracle" / "_ref" / "combined_sieve"
GAP_TEST = ROOT / "oracle" / "_ref" / "gap_test_simple"
OUT = Path(__file__).resolve().parent / "gaps.json"

# (name, p, d, mstart, minc, SL, max_prime_millions, sieve flags)
JOBS = [
    ("fn1", 907, 2190, 1, 200, 11000, 100, []),
    ("small_d7_odd", 509, 7, 31337, 2000, 3500, 10, []),
    ("small_bc_d30", 521, 30, 2024, 1500, 5000, 40, ["--bitcompressed"]),
    # SL close to 6P and many m: several sides run past the sieve length
    ("overflow_503_210", 503, 210, 1234567, 20000, 3024, 10, ["--rle"]),
]

GAP_LINE = re.compile(r"^(\d+)\s+([0-9.]+)\s+(\d+) \* (\d+)#/(\d+) -(\d+) to \+(\d+)$")
PRP_LINE = re.compile(r"prp tests (\d+)")


def run_job(p, d, mstart, minc, sl, mp, flags):
    with tempfile.TemporaryDirectory() as td:
        tdp = Path(td)
        (tdp / "unknowns").mkdir()
        args = [str(SIEVE), "-qqq", "--save-unknowns", "-p", str(p), "-d", str(d), "--mstart", str(mstart),
                "--minc", str(minc), "--max-prime", str(mp), "--sieve-length", str(sl), "-t", "1"] + flags
        # exits 1 after saving when there is no search database to record the range in
        subprocess.run(args, cwd=tdp, check=False, capture_output=True)
        files = list((tdp / "unknowns").iterdir())
        assert len(files) == 1, files
        data = files[0].read_bytes()
        out = subprocess.run([str(GAP_TEST), "-u", files[0].name, "--min-merit", "0", "-q"], cwd=tdp,
                             check=True, capture_output=True, text=True).stdout
    gaps = []
    for line in out.splitlines():
        g = GAP_LINE.match(line.strip())
        if g:
            gap, _, m, gp, gd, prev, nxt = g.groups()
            assert (int(gp), int(gd)) == (p, d) and int(gap) == int(prev) + int(nxt)
            gaps.append([int(m), int(prev), int(nxt)])
    prp = [int(x) for x in PRP_LINE.findall(out)]
    return files[0].name, hashlib.md5(data).hexdigest(), gaps, prp[-1]


def main():
    out = {}
    for name, p, d, mstart, minc, sl, mp, flags in JOBS:
        fn, md5, gaps, prp = run_job(p, d, mstart, minc, sl, mp, flags)
        compression = 1 if "--rle" in flags else 2 if "--bitcompressed" in flags else 0
        over = sum(1 for _, a, b in gaps if a > sl) + sum(1 for _, a, b in gaps if b > sl)
        sieve_goldens = json.loads((Path(__file__).resolve().parent / "goldens.json").read_text())
        if name in sieve_goldens:
            assert sieve_goldens[name]["md5"] == md5, name
        out[name] = {"p": p, "d": d, "mstart": mstart, "minc": minc, "sieve_length": sl,
                     "max_prime": mp * 1_000_000, "compression": compression, "unknowns_file": fn,
                     "unknowns_md5": md5, "prp_tests": prp, "past_sieve_length": over,
                     "source": "reference gap_test_simple run", "gaps": gaps}
        print(f"{name}: {len(gaps)} m, {prp} PRP tests, {over} sides past SL")
    OUT.write_text(json.dumps(out, separators=(",", ":")) + "\n")


if __name__ == "__main__":
    main()
