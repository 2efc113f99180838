"""ctypes binding of libpgsieve (C ABI declared in include/pgsieve.h).

Mirrors the reference's method2 entry point prime_gap_parallel
(combined_sieve.cpp:2014) as ``Sieve.method2(job) -> bytes`` (the unknowns
file contents) plus the number-theory primitives the sieve is built from.
The CUDA library is required: loading fails loudly when it is missing.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("PGSIEVE_LIB", PKG / "_build" / "libpgsieve.so"))
# tuned knobs per (device, job class), loaded into every context; empty
# PGSIEVE_TUNING turns it off, another path replaces it
TUNING_PATH = os.environ.get("PGSIEVE_TUNING", str(PKG / "tuning.tsv"))
HEADER = PKG.parent / "include" / "pgsieve.h"

PGS_OK = 0
PGS_EINVAL = -1
PGS_ENOMEM = -2
PGS_ECUDA = -3
PGS_EABORT = -4
PGS_ENODEV = -5
PGS_ETIMEOUT = -6

STAGES = ["setup", "primes", "kmod", "large", "rows", "text", "d2h", "spare"]


class PgsError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        super().__init__(f"pgsieve error {code}: {msg}")
        self.code = code


class Job(ctypes.Structure):
    _fields_ = [
        ("p", ctypes.c_uint32),
        ("d", ctypes.c_uint32),
        ("mstart", ctypes.c_uint64),
        ("minc", ctypes.c_uint64),
        ("sieve_length", ctypes.c_uint32),
        ("max_prime", ctypes.c_uint64),
        ("compression", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class Result(ctypes.Structure):
    _fields_ = [
        ("text", ctypes.POINTER(ctypes.c_char)),
        ("text_len", ctypes.c_uint64),
        ("rows", ctypes.c_uint64),
        ("primes", ctypes.c_uint64),
        ("prime_limit", ctypes.c_uint64),
        ("unknowns", ctypes.c_uint64),
        ("ms_total", ctypes.c_double),
        ("ms_stage", ctypes.c_double * 8),
        ("launches", ctypes.c_uint64),
        ("internal", ctypes.c_void_p),
    ]


class Plan(ctypes.Structure):
    _fields_ = [
        ("valid_ms", ctypes.c_uint64),
        ("coprime_x", ctypes.c_uint64),
        ("small_threshold", ctypes.c_uint64),
        ("medium_threshold", ctypes.c_uint64),
        ("prime_limit", ctypes.c_uint64),
        ("k_bits", ctypes.c_uint32),
        ("filename", ctypes.c_char * 256),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("failed", ctypes.c_uint64),
        ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double),
        ("mean_ms", ctypes.c_double),
        ("max_ms", ctypes.c_double),
        ("busy_s", ctypes.c_double),
        ("peak_bytes", ctypes.c_uint64),
        ("max_inflight", ctypes.c_uint64),
        ("host_prep_s", ctypes.c_double),
        ("host_fetch_s", ctypes.c_double),
        ("kmod_fills", ctypes.c_uint64),
        ("kmod_hits", ctypes.c_uint64),
        ("host_derive_s", ctypes.c_double),
        ("host_upload_s", ctypes.c_double),
        ("host_launch_s", ctypes.c_double),
        ("pinned_alloc_s", ctypes.c_double),
        ("pinned_allocs", ctypes.c_uint64),
        ("device_alloc_s", ctypes.c_double),
        ("device_allocs", ctypes.c_uint64),
    ]


class Unknowns(ctypes.Structure):
    _fields_ = [
        ("rows", ctypes.c_uint64),
        ("m", ctypes.POINTER(ctypes.c_uint64)),
        ("start", ctypes.POINTER(ctypes.c_uint64)),
        ("n_prev", ctypes.POINTER(ctypes.c_uint32)),
        ("n_next", ctypes.POINTER(ctypes.c_uint32)),
        ("dist", ctypes.POINTER(ctypes.c_uint32)),
        ("total", ctypes.c_uint64),
        ("internal", ctypes.c_void_p),
    ]


class GapParams(ctypes.Structure):
    _fields_ = [
        ("p", ctypes.c_uint32),
        ("d", ctypes.c_uint32),
        ("sieve_length", ctypes.c_uint32),
        ("min_merit", ctypes.c_float),
        ("one_side_skip", ctypes.c_int),
    ]


class GapResult(ctypes.Structure):
    _fields_ = [
        ("prev_p", ctypes.c_int32),
        ("next_p", ctypes.c_int32),
        ("p_tests", ctypes.c_uint32),
        ("n_tests", ctypes.c_uint32),
        ("flags", ctypes.c_uint32),
    ]


class Tuning(ctypes.Structure):
    """pgs_tuning: launch knobs per job class (output never depends on them)."""

    _fields_ = [
        ("direct_steps", ctypes.c_uint32),
        ("item_steps", ctypes.c_uint32),
        ("heavy_steps", ctypes.c_uint32),
        ("rows_per_cta", ctypes.c_uint32),
        ("text_chunks", ctypes.c_uint32),
        ("kmod_lsb_limbs", ctypes.c_uint32),
        ("large_form", ctypes.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class GapStats(ctypes.Structure):
    _fields_ = [
        ("rounds", ctypes.c_uint64),
        ("prp_tests", ctypes.c_uint64),
        ("limbs", ctypes.c_uint32),
    ]


@dataclass
class JobSpec:
    """Config fields of one method2 job; max_prime is absolute."""

    p: int
    d: int
    mstart: int
    minc: int
    sieve_length: int
    max_prime: int
    compression: int = 0

    def c(self) -> Job:
        return Job(self.p, self.d, self.mstart, self.minc, self.sieve_length, self.max_prime,
                   self.compression, 0)

    @property
    def filename(self) -> str:
        """Args::gen_unknown_fn (gap_common.cpp:732-749)."""
        return (f"{self.p}_{self.d}_{self.mstart}_{self.minc}_s{self.sieve_length}"
                f"_l{self.max_prime // 1_000_000}M.txt")


_u64p = ctypes.POINTER(ctypes.c_uint64)
_u32p = ctypes.POINTER(ctypes.c_uint32)

_SIGNATURES = {
    "pgs_version": (ctypes.c_char_p, []),
    "pgs_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "pgs_destroy": (None, [ctypes.c_void_p]),
    "pgs_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "pgs_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pgs_get_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "pgs_method2": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.POINTER(Result)]),
    "pgs_method1": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.POINTER(Result)]),
    "pgs_result_free": (None, [ctypes.POINTER(Result)]),
    "pgs_prepare": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.POINTER(ctypes.c_void_p)]),
    "pgs_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "pgs_fetch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Result)]),
    "pgs_prepared_free": (None, [ctypes.c_void_p]),
    "pgs_plan_job": (ctypes.c_int, [ctypes.POINTER(Job), ctypes.POINTER(Plan)]),
    "pgs_stage_ms": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double)]),
    "pgs_int_peak": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "pgs_primes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, _u64p,
                                  ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "pgs_k_mod_p": (ctypes.c_int, [ctypes.c_void_p, _u32p, ctypes.c_int, _u64p, ctypes.c_size_t, _u64p]),
    "pgs_modulo_search": (ctypes.c_int, [ctypes.c_void_p, _u64p, _u64p, _u64p, _u64p, _u64p,
                                         ctypes.c_size_t]),
    "pgs_large_hits": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                      ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, _u32p,
                                      _u64p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "pgs_large_hits_static": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                             ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, _u32p,
                                             _u64p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "pgs_fetch_unknowns": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Unknowns)]),
    "pgs_parse_unknowns": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.c_char_p,
                                          ctypes.c_uint64, ctypes.POINTER(Unknowns)]),
    "pgs_unknowns_free": (None, [ctypes.POINTER(Unknowns)]),
    "pgs_prp_test": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32,
                                    ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(ctypes.c_uint8)]),
    "pgs_prp_gaps": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(GapParams), ctypes.POINTER(Unknowns),
                                    ctypes.POINTER(GapResult), ctypes.POINTER(GapStats)]),
    "pgs_prp_gaps_prepared": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(GapParams),
                                             ctypes.POINTER(GapResult), ctypes.POINTER(GapStats)]),
    "pgs_table_reserve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "pgs_batch_prepare": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "pgs_batch_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_double)]),
    "pgs_batch_fetch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Result)]),
    "pgs_batch_free": (None, [ctypes.c_void_p]),
    "pgs_method2_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.c_int,
                                         ctypes.POINTER(Result)]),
    "pgs_server_start": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "pgs_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), _u64p]),
    "pgs_server_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(Result),
                                       ctypes.POINTER(ctypes.c_double)]),
    "pgs_server_stats_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ServerStats)]),
    "pgs_server_stop": (ctypes.c_int, [ctypes.c_void_p]),
    "pgs_tuning_default": (None, [ctypes.c_void_p]),
    "pgs_tuning_class": (ctypes.c_int, [ctypes.POINTER(Job), ctypes.c_char_p, ctypes.c_size_t]),
    "pgs_tuning_set": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.c_void_p]),
    "pgs_tuning_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.c_void_p]),
    "pgs_tuning_load": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "pgs_tuning_save": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "pgs_tune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.c_int, ctypes.c_void_p,
                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
}

_lib: ctypes.CDLL | None = None


def load(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Load libpgsieve.so (built by prime-gap_gb300/build.py)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"libpgsieve not built: {p} (run prime-gap_gb300/build.py)")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def header_symbols() -> list[str]:
    """Function names declared in include/pgsieve.h."""
    import re

    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(pgs_\w+)\s*\(", text, re.M)))


def plan(job: JobSpec) -> dict:
    lib = load()
    pl = Plan()
    rc = lib.pgs_plan_job(ctypes.byref(job.c()), ctypes.byref(pl))
    return {
        "rc": rc,
        "valid_ms": pl.valid_ms,
        "coprime_x": pl.coprime_x,
        "small_threshold": pl.small_threshold,
        "medium_threshold": pl.medium_threshold,
        "prime_limit": pl.prime_limit,
        "k_bits": pl.k_bits,
        "filename": pl.filename.decode(),
    }


def tuning_class(job: JobSpec) -> str:
    """The job's tuning class, P<p>.SL<log2 SL>.minc<log2 minc>.mp<log2 max_prime>."""
    buf = ctypes.create_string_buffer(64)
    n = load().pgs_tuning_class(ctypes.byref(job.c()), buf, 64)
    if n < 0:
        raise PgsError(n, "pgs_tuning_class")
    return buf.value.decode()


def tuning_default() -> dict:
    t = Tuning()
    load().pgs_tuning_default(ctypes.byref(t))
    return t.as_dict()


def _arr(ctype, values):
    a = (ctype * max(1, len(values)))()
    for i, v in enumerate(values):
        a[i] = v
    return a


class Sieve:
    """One library context on a CUDA device."""

    def __init__(self, device: int = 0, load_tuning: bool = True):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.pgs_create(device, ctypes.byref(h))
        if rc != PGS_OK:
            raise PgsError(rc, "pgs_create failed (no usable CUDA device?)")
        self.h = h
        if load_tuning and TUNING_PATH and Path(TUNING_PATH).exists():
            self.lib.pgs_tuning_load(self.h, str(TUNING_PATH).encode())

    # -- tuning (pgs_tuning_*, pgs_tune) --------------------------------------

    def tune(self, job: JobSpec, reps: int = 3) -> tuple[dict, float, float]:
        """Tune the job's class on this device: (knobs, ms with the
        defaults, ms with the knobs)."""
        t = Tuning()
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.pgs_tune(self.h, ctypes.byref(job.c()), reps, ctypes.byref(t), ctypes.byref(a),
                                      ctypes.byref(b)))
        return t.as_dict(), a.value, b.value

    def tuning_get(self, job: JobSpec) -> tuple[dict, bool]:
        t = Tuning()
        rc = self.lib.pgs_tuning_get(self.h, ctypes.byref(job.c()), ctypes.byref(t))
        if rc < 0:
            self._check(rc)
        return t.as_dict(), rc == 1

    def tuning_set(self, job: JobSpec, knobs: dict) -> None:
        t = Tuning(**{**tuning_default(), **knobs})
        self._check(self.lib.pgs_tuning_set(self.h, ctypes.byref(job.c()), ctypes.byref(t)))

    def tuning_load(self, path: str | os.PathLike) -> int:
        rc = self.lib.pgs_tuning_load(self.h, str(path).encode())
        if rc < 0:
            self._check(rc)
        return rc

    def tuning_save(self, path: str | os.PathLike) -> int:
        rc = self.lib.pgs_tuning_save(self.h, str(path).encode())
        if rc < 0:
            self._check(rc)
        return rc

    def close(self) -> None:
        if self.h:
            self.lib.pgs_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int) -> None:
        if rc != PGS_OK:
            raise PgsError(rc, self.lib.pgs_last_error(self.h).decode(errors="replace"))

    @property
    def stream(self) -> int:
        return self.lib.pgs_get_stream(self.h) or 0

    def set_stream(self, stream_ptr: int | None) -> None:
        self._check(self.lib.pgs_set_stream(self.h, stream_ptr))

    def method2(self, job: JobSpec, stats: dict | None = None) -> bytes:
        """Unknowns file bytes for one job (prime_gap_parallel + save)."""
        res = Result()
        self._check(self.lib.pgs_method2(self.h, ctypes.byref(job.c()), ctypes.byref(res)))
        try:
            data = ctypes.string_at(res.text, res.text_len)
            if stats is not None:
                stats.update(_result_stats(res))
        finally:
            self.lib.pgs_result_free(ctypes.byref(res))
        return data

    def method1(self, job: JobSpec, stats: dict | None = None) -> bytes:
        """The same bytes by the per-m path (pgs_method1, the reference's
        --method1 cross-check)."""
        res = Result()
        self._check(self.lib.pgs_method1(self.h, ctypes.byref(job.c()), ctypes.byref(res)))
        try:
            data = ctypes.string_at(res.text, res.text_len)
            if stats is not None:
                stats.update(_result_stats(res))
        finally:
            self.lib.pgs_result_free(ctypes.byref(res))
        return data

    def method2_view(self, job: JobSpec, stats: dict | None = None) -> "ResultView":
        """Like method2 but without copying: a view of the library-owned host
        buffer, valid until the returned object is closed."""
        res = Result()
        self._check(self.lib.pgs_method2(self.h, ctypes.byref(job.c()), ctypes.byref(res)))
        if stats is not None:
            stats.update(_result_stats(res))
        return ResultView(self.lib, res)

    def prepare(self, job: JobSpec) -> "Prepared":
        h = ctypes.c_void_p()
        self._check(self.lib.pgs_prepare(self.h, ctypes.byref(job.c()), ctypes.byref(h)))
        return Prepared(self, h, job)

    def reserve_table(self, limit: int) -> None:
        """Generate (once) the resident prime table up to ``limit``."""
        self._check(self.lib.pgs_table_reserve(self.h, limit))

    def batch(self, jobs: list[JobSpec], lanes: int = 8) -> "Batch":
        """Prepare many jobs over the resident prime table (pgs_batch_prepare)."""
        arr = (Job * len(jobs))(*[j.c() for j in jobs])
        h = ctypes.c_void_p()
        self._check(self.lib.pgs_batch_prepare(self.h, arr, len(jobs), lanes, ctypes.byref(h)))
        return Batch(self, h, len(jobs))

    def method2_batch(self, jobs: list[JobSpec]) -> list[bytes]:
        out = []
        for v in self.method2_batch_views(jobs):
            with v:
                out.append(v.bytes())
        return out

    def method2_batch_views(self, jobs: list[JobSpec]) -> list["ResultView"]:
        """pgs_method2_batch without copies: one view per job (close each)."""
        arr = (Job * len(jobs))(*[j.c() for j in jobs])
        res = (Result * len(jobs))()
        self._check(self.lib.pgs_method2_batch(self.h, arr, len(jobs), res))
        return [ResultView(self.lib, r) for r in res]

    def server(self, hbm_budget: int, lanes: int = 8) -> "Server":
        """Start the request server on this context (pgs_server_start)."""
        h = ctypes.c_void_p()
        self._check(self.lib.pgs_server_start(self.h, hbm_budget, lanes, ctypes.byref(h)))
        return Server(self, h)

    def parse_unknowns(self, job: JobSpec, text: bytes) -> dict:
        """Per-m unknown lists of an unknowns file, parsed on the device
        (numpy arrays m, start, n_prev, n_next, dist)."""
        u = Unknowns()
        self._check(self.lib.pgs_parse_unknowns(self.h, ctypes.byref(job.c()), text, len(text),
                                                ctypes.byref(u)))
        return _unknowns_out(self.lib, u)

    def prp_test(self, numbers: list[int]) -> list[bool]:
        """Base-2 strong probable-prime test of each number (pgs_prp_test)."""
        if not numbers:
            return []
        n_limbs = max(1, max((x.bit_length() + 31) // 32 for x in numbers))
        buf = (ctypes.c_uint32 * (n_limbs * len(numbers)))()
        for i, x in enumerate(numbers):
            for j in range(n_limbs):
                buf[i * n_limbs + j] = (x >> (32 * j)) & 0xFFFFFFFF
        out = (ctypes.c_uint8 * len(numbers))()
        self._check(self.lib.pgs_prp_test(self.h, buf, n_limbs, len(numbers), 1, out))
        return [bool(v) for v in out]

    def prp_gaps(self, p: int, d: int, sieve_length: int, lists: dict, min_merit: float = 18.0,
                 one_side_skip: bool = False) -> tuple[list[tuple[int, int, int, int, int]], dict]:
        """The gap around m*K for every row of ``lists`` (numpy arrays m, start,
        n_prev, n_next, dist as from parse_unknowns / Prepared.unknowns):
        [(prev_p, next_p, p_tests, n_tests, flags)] and the search stats."""
        import numpy as np

        rows = len(lists["m"])
        arrs = {k: np.ascontiguousarray(lists[k], dtype=t) for k, t in
                (("m", np.uint64), ("start", np.uint64), ("n_prev", np.uint32), ("n_next", np.uint32),
                 ("dist", np.uint32))}
        u = Unknowns()
        u.rows, u.total = rows, len(arrs["dist"])
        u.m = arrs["m"].ctypes.data_as(_u64p)
        u.start = arrs["start"].ctypes.data_as(_u64p)
        u.n_prev = arrs["n_prev"].ctypes.data_as(_u32p)
        u.n_next = arrs["n_next"].ctypes.data_as(_u32p)
        u.dist = arrs["dist"].ctypes.data_as(_u32p)
        prm = GapParams(p, d, sieve_length, min_merit, int(one_side_skip))
        out = (GapResult * max(1, rows))()
        st = GapStats()
        self._check(self.lib.pgs_prp_gaps(self.h, ctypes.byref(prm), ctypes.byref(u), out, ctypes.byref(st)))
        res = [(r.prev_p, r.next_p, r.p_tests, r.n_tests, r.flags) for r in out[:rows]]
        return res, {"rounds": st.rounds, "prp_tests": st.prp_tests, "limbs": st.limbs}

    def int_peak(self) -> float:
        """Measured 32-bit IMAD issue rate (per second)."""
        v = ctypes.c_double()
        self._check(self.lib.pgs_int_peak(self.h, ctypes.byref(v)))
        return v.value

    def primes(self, lo: int, hi: int) -> list[int]:
        n = ctypes.c_size_t()
        self._check(self.lib.pgs_primes(self.h, lo, hi, None, 0, ctypes.byref(n)))
        out = (ctypes.c_uint64 * max(1, n.value))()
        self._check(self.lib.pgs_primes(self.h, lo, hi, out, n.value, ctypes.byref(n)))
        return list(out[: n.value])

    def k_mod_p(self, limbs: list[int], q: list[int]) -> list[int]:
        out = (ctypes.c_uint64 * max(1, len(q)))()
        self._check(self.lib.pgs_k_mod_p(self.h, _arr(ctypes.c_uint32, limbs), len(limbs),
                                         _arr(ctypes.c_uint64, q), len(q), out))
        return list(out[: len(q)])

    def modulo_search(self, p, a, l, r) -> list[int]:
        n = len(p)
        out = (ctypes.c_uint64 * max(1, n))()
        self._check(self.lib.pgs_modulo_search(self.h, _arr(ctypes.c_uint64, p), _arr(ctypes.c_uint64, a),
                                               _arr(ctypes.c_uint64, l), _arr(ctypes.c_uint64, r), out, n))
        return list(out[:n])

    def large_hits(self, M: int, max_mi: int, SL: int, prime: int, base_r: int,
                   cap: int = 1 << 20) -> list[tuple[int, int]]:
        mi = (ctypes.c_uint32 * cap)()
        md = (ctypes.c_uint64 * cap)()
        n = ctypes.c_size_t()
        self._check(self.lib.pgs_large_hits(self.h, M, max_mi, SL, prime, base_r, mi, md, cap,
                                            ctypes.byref(n)))
        k = min(n.value, cap)
        return list(zip(mi[:k], md[:k]))


class ResultView:
    """Zero-copy access to a pgs_result's text (freed by close())."""

    def __init__(self, lib, res: Result):
        self.lib, self.res = lib, res
        self.view = (ctypes.c_char * res.text_len).from_address(
            ctypes.cast(res.text, ctypes.c_void_p).value or 0) if res.text_len else b""

    def __len__(self) -> int:
        return self.res.text_len

    def bytes(self) -> bytes:
        return bytes(self.view)

    def close(self) -> None:
        if self.res is not None:
            self.lib.pgs_result_free(ctypes.byref(self.res))
            self.res = None
            self.view = b""

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Prepared:
    """A job whose tables are resident on the device (pgs_prepare)."""

    def __init__(self, sieve: Sieve, h: ctypes.c_void_p, spec: JobSpec | None = None):
        self.sieve, self.h, self.spec = sieve, h, spec

    def run(self, record_stages: bool = True) -> None:
        self.sieve._check(self.sieve.lib.pgs_run(self.sieve.h, self.h, int(record_stages)))

    def stage_ms(self) -> tuple[dict, float]:
        out = (ctypes.c_double * 8)()
        tot = ctypes.c_double()
        self.sieve._check(self.sieve.lib.pgs_stage_ms(self.sieve.h, self.h, out, ctypes.byref(tot)))
        return {STAGES[i]: out[i] for i in range(8)}, tot.value

    def fetch(self, stats: dict | None = None) -> bytes:
        res = Result()
        self.sieve._check(self.sieve.lib.pgs_fetch(self.sieve.h, self.h, ctypes.byref(res)))
        try:
            data = ctypes.string_at(res.text, res.text_len)
            if stats is not None:
                stats.update(_result_stats(res))
        finally:
            self.sieve.lib.pgs_result_free(ctypes.byref(res))
        return data

    def prp_gaps(self, min_merit: float = 18.0, one_side_skip: bool = False):
        """The gap search over this job's lists in place on the device
        (pgs_prp_gaps_prepared): [(prev_p, next_p, p_tests, n_tests, flags)]
        per valid m and the search stats."""
        n = plan(self.spec)["valid_ms"]
        out = (GapResult * max(1, n))()
        st = GapStats()
        prm = GapParams(0, 0, 0, min_merit, int(one_side_skip))
        self.sieve._check(self.sieve.lib.pgs_prp_gaps_prepared(self.sieve.h, self.h, ctypes.byref(prm), out,
                                                                ctypes.byref(st)))
        return [(r.prev_p, r.next_p, r.p_tests, r.n_tests, r.flags) for r in out[:n]], \
            {"rounds": st.rounds, "prp_tests": st.prp_tests, "limbs": st.limbs}

    def unknowns(self) -> dict:
        """Per-m unknown lists of the last run, straight from the device."""
        u = Unknowns()
        self.sieve._check(self.sieve.lib.pgs_fetch_unknowns(self.sieve.h, self.h, ctypes.byref(u)))
        return _unknowns_out(self.sieve.lib, u)

    def close(self) -> None:
        if self.h:
            self.sieve.lib.pgs_prepared_free(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """Jobs prepared over the resident prime table; run as one CUDA graph."""

    def __init__(self, sieve: Sieve, h: ctypes.c_void_p, n: int):
        self.sieve, self.h, self.n = sieve, h, n

    def run(self, graph: bool = True) -> float:
        """Run every job; returns the batch's device time in ms."""
        ms = ctypes.c_double()
        self.sieve._check(self.sieve.lib.pgs_batch_run(self.sieve.h, self.h, int(graph), ctypes.byref(ms)))
        return ms.value

    def fetch_view(self, i: int) -> ResultView:
        res = Result()
        self.sieve._check(self.sieve.lib.pgs_batch_fetch(self.sieve.h, self.h, i, ctypes.byref(res)))
        return ResultView(self.sieve.lib, res)

    def fetch(self, i: int) -> bytes:
        with self.fetch_view(i) as v:
            return v.bytes()

    def close(self) -> None:
        if self.h:
            self.sieve.lib.pgs_batch_free(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Server:
    """Request server: jobs admitted in arrival order within an HBM budget."""

    def __init__(self, sieve: Sieve, h: ctypes.c_void_p):
        self.sieve, self.h = sieve, h

    def submit(self, job: JobSpec) -> int:
        t = ctypes.c_uint64()
        rc = self.sieve.lib.pgs_server_submit(self.h, ctypes.byref(job.c()), ctypes.byref(t))
        if rc != PGS_OK:
            raise PgsError(rc, "submit refused")
        return t.value

    def wait_view(self, ticket: int, timeout_ms: int = -1) -> tuple[ResultView, float]:
        res = Result()
        lat = ctypes.c_double()
        rc = self.sieve.lib.pgs_server_wait(self.h, ticket, timeout_ms, ctypes.byref(res), ctypes.byref(lat))
        if rc != PGS_OK:
            raise PgsError(rc, self.sieve.lib.pgs_last_error(self.sieve.h).decode(errors="replace"))
        return ResultView(self.sieve.lib, res), lat.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> tuple[bytes, float]:
        v, lat = self.wait_view(ticket, timeout_ms)
        with v:
            return v.bytes(), lat

    def stats(self) -> dict:
        st = ServerStats()
        self.sieve._check(self.sieve.lib.pgs_server_stats_get(self.h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def stop(self) -> None:
        if self.h:
            self.sieve.lib.pgs_server_stop(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()


def _result_stats(res: Result) -> dict:
    return {
        "text_len": res.text_len,
        "rows": res.rows,
        "primes": res.primes,
        "unknowns": res.unknowns,
        "prime_limit": res.prime_limit,
        "ms_total": res.ms_total,
        "ms_stage": {STAGES[i]: res.ms_stage[i] for i in range(8)},
        "launches": res.launches,
    }


def _unknowns_out(lib, u: Unknowns) -> dict:
    import numpy as np

    try:
        rows, total = u.rows, u.total
        arr = np.ctypeslib.as_array
        return {
            "m": arr(u.m, (max(rows, 1),))[:rows].copy(),
            "start": arr(u.start, (max(rows, 1),))[:rows].copy(),
            "n_prev": arr(u.n_prev, (max(rows, 1),))[:rows].copy(),
            "n_next": arr(u.n_next, (max(rows, 1),))[:rows].copy(),
            "dist": arr(u.dist, (max(total, 1),))[:total].copy(),
        }
    finally:
        lib.pgs_unknowns_free(ctypes.byref(u))
