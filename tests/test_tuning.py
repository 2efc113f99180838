"""The tuner's cache logic on the CPU: class keys, the cache file's line
format and its merge across devices (prime-gap_gb300/csrc/pg_tuning.h built
for the host), and the C ABI's class function and defaults."""
from __future__ import annotations

import ctypes

import pytest

import pgsieve


class _T(ctypes.Structure):
    _fields_ = pgsieve.Tuning._fields_


@pytest.fixture(scope="module")
def th(built):
    import build as pkg_build

    lib = ctypes.CDLL(str(pkg_build.TUNE_HOST_LIB))
    d = ctypes.c_double
    lib.th_put.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_T), d, d]
    lib.th_get.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_T),
                           ctypes.POINTER(d)]
    lib.th_parse.argtypes = [ctypes.c_char_p, ctypes.POINTER(_T)]
    lib.th_class.argtypes = [ctypes.POINTER(pgsieve.Job), ctypes.c_char_p, ctypes.c_size_t]
    return lib


def _knobs(**kw):
    return _T(**{**pgsieve.tuning_default(), **kw})


def test_class_keys(th, built):
    cases = [(pgsieve.JobSpec(1511, 2190, 12345679, 100000, 20000, 2_000_000_000), "P1511.SL14.minc16.mp30"),
             (pgsieve.JobSpec(503, 210, 1, 10000, 5000, 100_000_000), "P503.SL12.minc13.mp26"),
             (pgsieve.JobSpec(3001, 2190, 1, 1, 40000, 10**10), "P3001.SL15.minc0.mp33"),
             (pgsieve.JobSpec(907, 2190, 1, 200, 11000, 10**8), "P907.SL13.minc7.mp26")]
    buf = ctypes.create_string_buffer(64)
    for job, want in cases:
        assert pgsieve.tuning_class(job) == want
        assert th.th_class(ctypes.byref(job.c()), buf, 64) == len(want) and buf.value.decode() == want
    # the class ignores mstart, d and compression, and max_prime below the next power of two
    a = pgsieve.JobSpec(1511, 2190, 7, 70000, 17000, 2**31 + 1, 2)
    b = pgsieve.JobSpec(1511, 1, 10**8, 65536, 16384, 4 * 10**9, 0)
    assert pgsieve.tuning_class(a) == pgsieve.tuning_class(b)
    c = pgsieve.JobSpec(1511, 1, 10**8, 65536, 16384, 2**31 - 1, 0)
    assert pgsieve.tuning_class(c) != pgsieve.tuning_class(b)


def test_committed_table_covers_the_configs(th, built):
    """The shipped GB300 table parses under the current class format and has
    an entry for each of configs 1-3 (the classes the bench's jobs look up)."""
    from pathlib import Path

    table = str(Path(pgsieve.__file__).resolve().parent / "tuning.tsv").encode()
    out, ms = _T(), (ctypes.c_double * 2)()
    for job in (pgsieve.JobSpec(503, 210, 1234567, 10000, 5000, 100_000_000),
                pgsieve.JobSpec(1511, 2190, 12345679, 100000, 20000, 2_000_000_000),
                pgsieve.JobSpec(3001, 2190, 123457, 100000, 40000, 10**10)):
        cls = pgsieve.tuning_class(job).encode()
        assert th.th_get(table, b"NVIDIA GB300", cls, ctypes.byref(out), ms) == 1, cls


def test_defaults_are_the_built_in_constants(built):
    assert pgsieve.tuning_default() == {"direct_steps": 24, "item_steps": 64, "heavy_steps": 4096,
                                        "rows_per_cta": 16, "text_chunks": 4, "kmod_lsb_limbs": 32,
                                        "large_form": 0}


def test_cache_file_round_trip_and_device_merge(th, tmp_path):
    f = str(tmp_path / "tuning.tsv").encode()
    out, ms = _T(), (ctypes.c_double * 2)()
    assert th.th_get(f, b"NVIDIA GB300", b"P1511.SL14.minc16.mp30", ctypes.byref(out), ms) == -1  # no file yet
    assert th.th_put(f, b"NVIDIA GB300", b"P1511.SL14.minc16.mp30", ctypes.byref(_knobs(heavy_steps=8192)), 10.2, 9.9) == 1
    assert th.th_put(f, b"NVIDIA B200", b"P1511.SL14.minc16.mp30", ctypes.byref(_knobs(item_steps=32)), 12.0, 11.0) == 1
    assert th.th_put(f, b"NVIDIA GB300", b"P503.SL12.minc13.mp26", ctypes.byref(_knobs(rows_per_cta=8)), 1.0, 0.9) == 2
    assert th.th_get(f, b"NVIDIA GB300", b"P1511.SL14.minc16.mp30", ctypes.byref(out), ms) == 1
    assert (out.heavy_steps, out.item_steps, tuple(ms)) == (8192, 64, (10.2, 9.9))
    assert th.th_get(f, b"NVIDIA B200", b"P1511.SL14.minc16.mp30", ctypes.byref(out), ms) == 1
    assert (out.heavy_steps, out.item_steps) == (4096, 32)
    assert th.th_get(f, b"NVIDIA GB300", b"P503.SL12.minc13.mp26", ctypes.byref(out), ms) == 1
    assert out.rows_per_cta == 8
    assert th.th_get(f, b"NVIDIA GB300", b"P999.SL1.minc1", ctypes.byref(out), ms) == 0
    lines = (tmp_path / "tuning.tsv").read_text().splitlines()
    assert lines[0].startswith("#") and len(lines) == 4


@pytest.mark.parametrize("line,ok", [
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 64 4096 16 4 32 0\t10 9", True),
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 64 4096 16 4 32 1", True),
    ("# comment", False),
    ("", False),
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 48 4096 16 4 32 0", False),   # item_steps not a power 32..128
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 64 4096 33 4 32 0", False),   # rows_per_cta > 32
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 64 4096 16 5 32 0", False),   # text_chunks > 4
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 64 16 16 4 32 0", False),     # heavy below direct / 256
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 64 4096 16 4 32 2", True),    # pooled, K mod p inside (32-bit)
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 64 4096 16 4 32 7", True),    # warps alone, K mod p inside
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 64 4096 16 4 32 8", False),   # no fourth form bit
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 64 4096 16 4 32", False),     # a line of the six-knob format
    ("NVIDIA GB300\tP1511.SL14.minc16.mp30\t24 64 4096", False),             # short
    ("NVIDIA GB300 P1511.SL14.minc16.mp30 24 64 4096 16 4 32 0", False),       # no tabs
])
def test_cache_line_validation(th, line, ok):
    out = _T()
    assert th.th_parse(line.encode(), ctypes.byref(out)) == int(ok)
