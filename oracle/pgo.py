"""ORACLE -- test infrastructure only.

ctypes binding of the C restatement of the reference's method2 sieve
(oracle/m2_oracle.c).  Only tests, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use it, and only as the checker.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libm2oracle.so"
BIN_PATH = HERE / "_build" / "m2_oracle"


class OJob(ctypes.Structure):
    _fields_ = [
        ("p", ctypes.c_uint32),
        ("d", ctypes.c_uint32),
        ("mstart", ctypes.c_uint64),
        ("minc", ctypes.c_uint64),
        ("sieve_length", ctypes.c_uint32),
        ("max_prime", ctypes.c_uint64),
        ("compression", ctypes.c_int32),
        ("threads", ctypes.c_int32),
    ]


class OPlan(ctypes.Structure):
    _fields_ = [
        ("small_threshold", ctypes.c_uint64),
        ("medium_threshold", ctypes.c_uint64),
        ("last_prime", ctypes.c_uint64),
        ("valid_ms", ctypes.c_uint64),
        ("coprime_x", ctypes.c_uint64),
        ("prime_limit", ctypes.c_uint64),
    ]


class OLists(ctypes.Structure):
    _fields_ = [
        ("rows", ctypes.c_uint64),
        ("m", ctypes.POINTER(ctypes.c_uint64)),
        ("n_prev", ctypes.POINTER(ctypes.c_uint32)),
        ("n_next", ctypes.POINTER(ctypes.c_uint32)),
        ("start", ctypes.POINTER(ctypes.c_uint64)),
        ("dist", ctypes.POINTER(ctypes.c_uint32)),
        ("total", ctypes.c_uint64),
    ]


_lib = None
_u64p = ctypes.POINTER(ctypes.c_uint64)


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise FileNotFoundError(f"oracle not built: {LIB_PATH}")
        lib = ctypes.CDLL(str(LIB_PATH))
        lib.pgo_method2.argtypes = [ctypes.POINTER(OJob), ctypes.POINTER(ctypes.c_void_p),
                                    ctypes.POINTER(ctypes.c_size_t)]
        lib.pgo_method2.restype = ctypes.c_int
        lib.pgo_free.argtypes = [ctypes.c_void_p]
        lib.pgo_modulo_search_euclid_small.restype = ctypes.c_uint32
        lib.pgo_modulo_search_euclid_small.argtypes = [ctypes.c_uint32] * 4
        lib.pgo_modulo_search_euclid.restype = ctypes.c_uint64
        lib.pgo_modulo_search_euclid.argtypes = [ctypes.c_uint64] * 4
        lib.pgo_modulo_search_euclid_stack.restype = ctypes.c_uint64
        lib.pgo_modulo_search_euclid_stack.argtypes = [ctypes.c_uint64] * 4
        lib.pgo_modulo_search_all_large.restype = ctypes.c_size_t
        lib.pgo_modulo_search_all_large.argtypes = [
            ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
            ctypes.POINTER(ctypes.c_uint32), _u64p, ctypes.c_size_t]
        lib.pgo_build_k.restype = ctypes.c_int
        lib.pgo_build_k.argtypes = [ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.POINTER(ctypes.c_uint32), ctypes.c_int]
        lib.pgo_k_mod.restype = ctypes.c_uint64
        lib.pgo_k_mod.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_int, ctypes.c_uint64]
        lib.pgo_primes.restype = ctypes.c_size_t
        lib.pgo_primes.argtypes = [ctypes.c_uint64, ctypes.c_uint64, _u64p, ctypes.c_size_t]
        lib.pgo_plan_job.restype = ctypes.c_int
        lib.pgo_plan_job.argtypes = [ctypes.POINTER(OJob), ctypes.POINTER(OPlan)]
        lib.pgo_trial_division.restype = ctypes.c_int
        lib.pgo_trial_division.argtypes = [ctypes.POINTER(OJob), _u64p,
                                           ctypes.POINTER(ctypes.c_int64), ctypes.c_size_t, _u64p]
        lib.pgo_parse_unknowns.restype = ctypes.c_int
        lib.pgo_parse_unknowns.argtypes = [ctypes.POINTER(OJob), ctypes.c_char_p, ctypes.c_size_t,
                                           ctypes.POINTER(OLists)]
        lib.pgo_method2_lists.restype = ctypes.c_int
        lib.pgo_method2_lists.argtypes = [ctypes.POINTER(OJob), ctypes.POINTER(OLists)]
        lib.pgo_lists_free.argtypes = [ctypes.POINTER(OLists)]
        _lib = lib
    return _lib


def _job(p, d, mstart, minc, sieve_length, max_prime, compression=0, threads=1) -> OJob:
    return OJob(p, d, mstart, minc, sieve_length, max_prime, compression, threads)


def method2(p, d, mstart, minc, sieve_length, max_prime, compression=0, threads=1) -> bytes:
    """Unknowns file bytes from the CPU restatement (max_prime absolute)."""
    lib = load()
    buf = ctypes.c_void_p()
    n = ctypes.c_size_t()
    rc = lib.pgo_method2(ctypes.byref(_job(p, d, mstart, minc, sieve_length, max_prime,
                                           compression, threads)), ctypes.byref(buf), ctypes.byref(n))
    if rc != 0:
        raise RuntimeError(f"oracle failed with {rc}")
    try:
        return ctypes.string_at(buf, n.value)
    finally:
        lib.pgo_free(buf)


def plan(p, d, mstart, minc, sieve_length, max_prime) -> dict:
    lib = load()
    pl = OPlan()
    rc = lib.pgo_plan_job(ctypes.byref(_job(p, d, mstart, minc, sieve_length, max_prime)),
                          ctypes.byref(pl))
    return {"rc": rc, "small_threshold": pl.small_threshold, "medium_threshold": pl.medium_threshold,
            "last_prime": pl.last_prime, "valid_ms": pl.valid_ms, "coprime_x": pl.coprime_x,
            "prime_limit": pl.prime_limit}


def build_k(p: int, d: int) -> list[int]:
    lib = load()
    buf = (ctypes.c_uint32 * 8192)()
    n = lib.pgo_build_k(p, d, buf, 8192)
    if n < 0:
        raise ValueError(f"bad K ({n})")
    return list(buf[:n])


def k_mod(limbs: list[int], q: int) -> int:
    lib = load()
    arr = (ctypes.c_uint32 * len(limbs))(*limbs)
    return lib.pgo_k_mod(arr, len(limbs), q)


def primes(lo: int, hi: int) -> list[int]:
    lib = load()
    n = lib.pgo_primes(lo, hi, None, 0)
    out = (ctypes.c_uint64 * max(1, n))()
    lib.pgo_primes(lo, hi, out, n)
    return list(out[:n])


def modulo_search(p, a, l, r) -> int:
    return load().pgo_modulo_search_euclid(p, a, l, r)


def modulo_search_stack(p, a, l, r) -> int:
    return load().pgo_modulo_search_euclid_stack(p, a, l, r)


def all_large(M, max_mi, SL, prime, base_r, cap=1 << 20) -> list[tuple[int, int]]:
    lib = load()
    mi = (ctypes.c_uint32 * cap)()
    md = (ctypes.c_uint64 * cap)()
    n = lib.pgo_modulo_search_all_large(M, max_mi, SL, prime, base_r, mi, md, cap)
    k = min(n, cap)
    return list(zip(mi[:k], md[:k]))


def all_large_count(M, max_mi, SL, prime, base_r) -> int:
    """Number of hits of modulo_search_euclid_all_large (none stored)."""
    lib = load()
    mi = (ctypes.c_uint32 * 1)()
    md = (ctypes.c_uint64 * 1)()
    return int(lib.pgo_modulo_search_all_large(M, max_mi, SL, prime, base_r, mi, md, 0))


def trial_division(job: dict, ms: list[int], xs: list[int], threads=8) -> list[int]:
    """Smallest prime <= the sieve limit dividing m*K + X, or 0."""
    lib = load()
    n = len(ms)
    out = (ctypes.c_uint64 * max(1, n))()
    m_arr = (ctypes.c_uint64 * max(1, n))(*ms)
    x_arr = (ctypes.c_int64 * max(1, n))(*xs)
    rc = lib.pgo_trial_division(ctypes.byref(_job(threads=threads, **job)), m_arr, x_arr, n, out)
    if rc != 0:
        raise RuntimeError(f"trial division failed {rc}")
    return list(out[:n])


def _lists_out(lib, rc, ol: OLists) -> dict:
    import numpy as np

    if rc != 0:
        raise RuntimeError(f"oracle lists failed: {rc}")
    try:
        rows, total = ol.rows, ol.total
        return {
            "m": np.ctypeslib.as_array(ol.m, (max(rows, 1),))[:rows].copy(),
            "n_prev": np.ctypeslib.as_array(ol.n_prev, (max(rows, 1),))[:rows].copy(),
            "n_next": np.ctypeslib.as_array(ol.n_next, (max(rows, 1),))[:rows].copy(),
            "start": np.ctypeslib.as_array(ol.start, (max(rows, 1),))[:rows].copy(),
            "dist": np.ctypeslib.as_array(ol.dist, (max(total, 1),))[:total].copy(),
        }
    finally:
        lib.pgo_lists_free(ctypes.byref(ol))


def method2_lists(p, d, mstart, minc, sieve_length, max_prime, threads=1) -> dict:
    """Unknowns per valid m as arrays (m, n_prev, n_next, start, dist)."""
    lib = load()
    ol = OLists()
    rc = lib.pgo_method2_lists(ctypes.byref(_job(p, d, mstart, minc, sieve_length, max_prime, 0,
                                                 threads)), ctypes.byref(ol))
    return _lists_out(lib, rc, ol)


def parse_unknowns(p, d, mstart, minc, sieve_length, max_prime, compression, text: bytes) -> dict:
    """parse_unknown_line over a whole unknowns file (any compression)."""
    lib = load()
    ol = OLists()
    rc = lib.pgo_parse_unknowns(ctypes.byref(_job(p, d, mstart, minc, sieve_length, max_prime,
                                                  compression)), text, len(text), ctypes.byref(ol))
    return _lists_out(lib, rc, ol)
