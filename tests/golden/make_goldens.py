"""Regenerate tests/golden/goldens.json from the reference itself.

Runs the reference combined_sieve compiled from its own sources by
oracle/build_ref.sh (oracle/_ref/combined_sieve, or the wheel-fixed copy for
jobs the unmodified reference aborts on) with one thread and records the md5
and size of each unknowns file.  One thread because the reference's
multi-threaded medium-prime phase can lose marks to a data race (threads
read-modify-write the same vector<bool> word, combined_sieve.cpp:2282-2290),
which shows up as extra unknowns: misc/tests.sh's FN2 hashes to
540add3a... instead of a8d85c96... with -t 8 on an 8-core host.  Entries marked "published" carry md5 values printed in the
reference's own test script / docs; the script checks they still reproduce.

    python tests/golden/make_goldens.py [--with-large]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import sqlite3
import subprocess
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
REF_DIR = Path("/root/reference")
REF_BIN = ROOT / "oracle" / "_ref" / "combined_sieve"
REF_FIX = ROOT / "oracle" / "_ref" / "combined_sieve_wheelfix"
OUT = Path(__file__).resolve().parent / "goldens.json"

# (name, p, d, mstart, minc, SL, max_prime_millions, flags, published md5 or None, source)
JOBS = [
    ("fn1", 907, 2190, 1, 200, 11000, 100, [], "15a5cbff7301262caf047028c05f0525", "misc/tests.sh:66"),
    ("fn1_rle", 907, 2190, 1, 200, 11000, 100, ["--rle"], "2ed7b0b9621dab602f204865360a3c56", "misc/tests.sh:85"),
    ("fn1_bitcompressed", 907, 2190, 1, 200, 11000, 100, ["--bitcompressed"],
     "6edd5f50c4f588890a168461a7240c47", "misc/tests.sh:94"),
    ("fn2", 953, 1, 1, 10000, 8000, 20, [], "a8d85c965ddf2d9601e93c9920a9aa12", "misc/tests.sh:71"),
    ("ext_907_210", 907, 210, 1, 1000, 7554, 1000, [], "d74bd47c8d43eac9a2309fc7722839ac", "EXTENDED.md:186-187"),
    # reference runs in this container (seeded stand-ins for the benchmark configs)
    ("config1", 503, 210, 1234567, 10000, 5000, 100, [], None, "reference run"),
    ("small_d1", 503, 1, 987654, 3000, 4000, 30, [], None, "reference run"),
    ("small_d2", 601, 2, 55555, 2500, 4000, 20, [], None, "reference run"),
    ("small_d30", 701, 30, 777777, 3000, 6000, 50, [], None, "reference run"),
    ("small_d2190", 1009, 2190, 4242, 4000, 8000, 200, [], None, "reference run"),
    ("small_d30030", 797, 30030, 123, 20000, 9000, 150, [], None, "reference run"),
    ("small_d7_odd", 509, 7, 31337, 2000, 3500, 10, [], None, "reference run"),
    ("small_d73_sl_odd", 557, 73, 1000003, 1500, 4001, 40, [], None, "reference run"),
    ("small_rle_d210", 503, 210, 9999, 2000, 5000, 60, ["--rle"], None, "reference run"),
    ("small_bc_d30", 521, 30, 2024, 1500, 5000, 40, ["--bitcompressed"], None, "reference run"),
    ("edge_maxprime_1M", 503, 210, 1, 1000, 5000, 1, [], None, "reference run"),
]
LARGE_JOBS = [
    ("config2", 1511, 2190, 12345679, 100000, 20000, 2000, [], None, "reference run"),
]


def run_ref(binary: Path, p, d, mstart, minc, sl, mp, flags, threads=1) -> tuple[bytes, float]:
    with tempfile.TemporaryDirectory() as td:
        tdp = Path(td)
        (tdp / "unknowns").mkdir()
        db = tdp / "test.db"
        con = sqlite3.connect(db)
        con.executescript((REF_DIR / "schema.sql").read_text())
        con.commit()
        con.close()
        cmd = [str(binary), "-qqq", "--save", "-p", str(p), "-d", str(d), "--mstart", str(mstart),
               "--minc", str(minc), "--sieve-length", str(sl), "--max-prime", str(mp),
               "--search-db", str(db), "-t", str(threads), *flags]
        t = time.perf_counter()
        subprocess.run(cmd, cwd=td, check=True, capture_output=True)
        dt = time.perf_counter() - t
        files = list((tdp / "unknowns").iterdir())
        assert len(files) == 1, files
        return files[0].read_bytes(), dt


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--with-large", action="store_true")
    a = ap.parse_args()
    jobs = JOBS + (LARGE_JOBS if a.with_large else [])
    old = json.loads(OUT.read_text()) if OUT.exists() else {}
    out = {}
    for name, p, d, ms, mi, sl, mp, flags, published, source in jobs:
        data, dt = run_ref(REF_BIN, p, d, ms, mi, sl, mp, flags)
        md5 = hashlib.md5(data).hexdigest()
        if published:
            assert md5 == published, (name, md5, published)
        out[name] = {
            "p": p, "d": d, "mstart": ms, "minc": mi, "sieve_length": sl,
            "max_prime": mp * 1_000_000, "compression": 1 if "--rle" in flags else 2 if "--bitcompressed" in flags else 0,
            "md5": md5, "bytes": len(data), "source": source, "ref_seconds_1t": round(dt, 3),
        }
        print(f"{name:22s} {md5} {len(data):>10d} B {dt:7.2f} s")
    for k, v in old.items():
        out.setdefault(k, v)
    OUT.write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
