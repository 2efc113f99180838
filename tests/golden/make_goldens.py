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

With --mix it writes tests/golden/mix_goldens.json instead: the reference's
md5 for every job of the seeded 64-job mix (workloads.mixed_jobs(64, seed=4))
and for jobs whose primes cross 2^32, run as concurrent one-thread reference
processes.  Jobs with gcd(d, 210) = 30 and SL > 30,583 go through the
wheel-fixed copy, because the unmodified reference aborts on them
(combined_sieve.cpp:1229); its bytes equal the unmodified --method1 output
(checked on config 3, golden 1781f036...).

    python tests/golden/make_goldens.py [--with-large] [--mix] [-j 8]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import json
import math
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
REF_BIN = ROOT / "oracle" / "_ref" / "combined_sieve"
REF_FIX = ROOT / "oracle" / "_ref" / "combined_sieve_wheelfix"
OUT = Path(__file__).resolve().parent / "goldens.json"
MIX_OUT = Path(__file__).resolve().parent / "mix_goldens.json"

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
    # m past 2^32 (64-bit m in the walk starts, the row residues and the text),
    # up to the reference's limit mstart + minc <= 1e10 + 1
    ("big_m_cross_2e32", 503, 210, 4294965796, 3000, 5000, 100, [], None, "reference run"),
    ("big_m_1e10_d7_odd", 509, 7, 9999997000, 3000, 3500, 10, [], None, "reference run"),
    ("big_m_rle_d2190", 907, 2190, 6000000001, 2000, 11000, 100, ["--rle"], None, "reference run"),
    ("big_m_bc_d30", 521, 30, 8589934000, 1500, 5000, 40, ["--bitcompressed"], None, "reference run"),
]
LARGE_JOBS = [
    ("config2", 1511, 2190, 12345679, 100000, 20000, 2000, [], None, "reference run"),
]

# Jobs whose sieving primes cross 2^32 (64-bit K mod p and walk starts):
# (name, p, d, mstart, minc, SL, max_prime_millions, flags)
WIDE_JOBS = [
    ("w64_503_210", 503, 210, 1234567, 300, 5000, 4400, []),
    ("w64_1009_2190_rle", 1009, 2190, 777, 200, 9000, 4300, ["--rle"]),
    ("w64_797_30030", 797, 30030, 5550001, 3000, 11500, 6000, []),
    ("w64_1511_1_bc", 1511, 1, 424242, 1500, 23500, 5000, ["--bitcompressed"]),
    ("w64_2003_2190", 2003, 2190, 31415926, 2000, 32000, 8000, []),
    ("w64_3001_210", 3001, 210, 2718281, 1000, 40000, 12000, []),
    ("w64_1009_2", 1009, 2, 99991, 2500, 15000, 5000, []),
    ("w64_601_7", 601, 7, 8675309, 1200, 6500, 4500, []),
]


def run_ref(binary: Path, p, d, mstart, minc, sl, mp, flags, threads=1) -> tuple[bytes, float]:
    with tempfile.TemporaryDirectory() as td:
        tdp = Path(td)
        (tdp / "unknowns").mkdir()
        cmd = [str(binary), "-qqq", "--save", "-p", str(p), "-d", str(d), "--mstart", str(mstart),
               "--minc", str(minc), "--sieve-length", str(sl), "--max-prime", str(mp),
               "-t", str(threads), *flags]
        t = time.perf_counter()
        # exits 1 after saving the file when there is no search database to record the range in
        subprocess.run(cmd, cwd=td, check=False, capture_output=True)
        dt = time.perf_counter() - t
        files = list((tdp / "unknowns").iterdir())
        assert len(files) == 1, files
        return files[0].read_bytes(), dt


def _needs_wheelfix(d: int, sl: int) -> bool:
    """The unmodified reference aborts for gcd(d, 210) = 30 and SL > 30,583."""
    return math.gcd(d, 210) == 30 and sl > 30583


def _mix_entry(job) -> dict:
    name, p, d, ms, mi, sl, mp, flags, source = job
    binary = REF_FIX if _needs_wheelfix(d, sl) else REF_BIN
    data, dt = run_ref(binary, p, d, ms, mi, sl, mp, flags)
    return {
        "name": name, "p": p, "d": d, "mstart": ms, "minc": mi, "sieve_length": sl,
        "max_prime": mp * 1_000_000,
        "compression": 1 if "--rle" in flags else 2 if "--bitcompressed" in flags else 0,
        "md5": hashlib.md5(data).hexdigest(), "bytes": len(data),
        "source": source + (" (wheel-fixed copy)" if binary == REF_FIX else ""),
        "ref_seconds_1t": round(dt, 3),
    }


def make_mix(workers: int) -> None:
    sys.path.insert(0, str(ROOT / "prime-gap_gb300"))
    import workloads

    jobs = []
    for i, j in enumerate(workloads.mixed_jobs(64, seed=4)):
        assert j.max_prime % 1_000_000 == 0 and j.compression == 0
        jobs.append((f"mix64_{i:02d}", j.p, j.d, j.mstart, j.minc, j.sieve_length, j.max_prime // 1_000_000,
                     [], "reference run, workloads.mixed_jobs(64, seed=4)"))
    jobs += [(*w, "reference run, primes past 2^32") for w in WIDE_JOBS]
    # longest first so the pool's tail is short
    jobs.sort(key=lambda t: -(t[4] * t[5] * math.log(t[6]) + 30 * t[6] * t[1] / 1000))
    out = {}
    with cf.ProcessPoolExecutor(max_workers=workers) as ex:
        for e in ex.map(_mix_entry, jobs):
            out[e.pop("name")] = e
            print(f"{len(out):3d}/{len(jobs)} {e['md5']} {e['bytes']:>10d} B {e['ref_seconds_1t']:8.2f} s",
                  flush=True)
    ordered = {k: out[k] for k in sorted(out)}
    MIX_OUT.write_text(json.dumps(ordered, indent=1) + "\n")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--with-large", action="store_true")
    ap.add_argument("--mix", action="store_true")
    ap.add_argument("-j", type=int, default=8)
    a = ap.parse_args()
    if a.mix:
        make_mix(a.j)
        return
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
