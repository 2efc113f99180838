"""The drop-in combined_sieve CLI end to end on the device: the reference's
misc/tests.sh FN1 invocations write byte-identical unknowns files (plain,
--rle, --bitcompressed) and record the run in the search database's `range`
table like insert_range_db (combined_sieve.cpp:347-380)."""
from __future__ import annotations

import hashlib
import sqlite3
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "prime-gap_gb300" / "_build" / "combined_sieve"
FN1 = "-p 907 -d 2190 --mstart 1 --minc 200 --max-prime 100 --sieve-length 11000 --save-unknowns -qqq"


def _db(path: Path) -> Path:
    """A search database with the `range` columns insert_range_db writes."""
    db = path / "search.db"
    con = sqlite3.connect(db)
    con.execute("CREATE TABLE range(rid INTEGER PRIMARY KEY, P INTEGER, D INTEGER, m_start INTEGER,"
                " m_inc INTEGER, sieve_length INTEGER, max_prime INTEGER, min_merit REAL, num_m INTEGER,"
                " time_sieve REAL)")
    con.commit()
    con.close()
    return db


@pytest.mark.parametrize("flag,golden", [("", "fn1"), ("--rle", "fn1_rle"),
                                         ("--bitcompressed", "fn1_bitcompressed")])
def test_cli_writes_reference_file_and_range_row(built, goldens, tmp_path, flag, golden):
    (tmp_path / "unknowns").mkdir()
    db = _db(tmp_path)
    args = [str(CLI), *FN1.split(), *flag.split(), "--search-db", str(db)]
    p = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    files = list((tmp_path / "unknowns").iterdir())
    assert [f.name for f in files] == ["907_2190_1_200_s11000_l100M.txt"], p.stdout
    assert hashlib.md5(files[0].read_bytes()).hexdigest() == goldens[golden]["md5"]
    if "libsqlite3.so.0 not available" in p.stdout:
        pytest.skip("no libsqlite3 on this host: file checked, range row not")
    assert p.returncode == 0, p.stdout
    rows = sqlite3.connect(db).execute("SELECT P, D, m_start, m_inc, sieve_length, max_prime, num_m FROM range")
    assert rows.fetchall() == [(907, 2190, 1, 200, 11000, 100_000_000, 53)]
    # a second run refuses to overwrite the file (combined_sieve.cpp:121-126)
    p2 = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert p2.returncode == 1 and "already exists" in p2.stdout
