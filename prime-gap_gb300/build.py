"""Build recipe for libpgsieve (CUDA, sm_103a), the combined_sieve CLI and the
oracle / test helpers.  Everything is built in-tree under ``_build`` folders;
translation units compile in parallel.

    python prime-gap_gb300/build.py            # everything
    python prime-gap_gb300/build.py --lib      # libpgsieve.so + CLI only
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"
ORACLE_BUILD = ORACLE / "_build"
TESTS_NATIVE = ROOT / "tests" / "native"

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
    f"-I{INCLUDE}", f"-I{CSRC}",
]
CU_SOURCES = ["pg_primes.cu", "pg_kmod.cu", "pg_large.cu", "pg_rows.cu", "pg_tools.cu", "pg_host.cu",
              "pg_api.cu", "pg_batch.cu", "pg_static.cu", "pg_unknowns.cu", "pg_prp.cu", "pg_tune.cu"]

LIB = BUILD / "libpgsieve.so"
CLI = BUILD / "combined_sieve"
GAP_TEST_CLI = BUILD / "gap_test"
ORACLE_LIB = ORACLE_BUILD / "libm2oracle.so"
ORACLE_BIN = ORACLE_BUILD / "m2_oracle"
ARITH_HOST_LIB = BUILD / "libpgarith_host.so"
TUNE_HOST_LIB = BUILD / "libpgtune_host.so"


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n"
                           f"{proc.stdout}\n{proc.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def build_lib(jobs: int = 8, verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    objs = []
    todo = []
    hdrs = _headers()
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            todo.append([NVCC, *NVCC_FLAGS, "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for cmd, fut in [(c, ex.submit(_run, c)) for c in todo]:
            if verbose:
                print(" ".join(cmd))
            fut.result()
    if _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-cudart", "static"])
    for src, out in ((HOST / "combined_sieve.cpp", CLI), (HOST / "gap_test.cpp", GAP_TEST_CLI)):
        if src.exists() and _stale(out, [src, HOST / "cli_common.h", LIB] + hdrs):
            _run(["g++", "-O2", "-std=c++17", "-Wall", f"-I{INCLUDE}", str(src), "-o", str(out),
                  f"-L{BUILD}", "-lpgsieve", "-Wl,-rpath,$ORIGIN", "-ldl"])
    return LIB


def build_oracle() -> Path:
    """The oracle is test infrastructure (checker only)."""
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    src = ORACLE / "m2_oracle.c"
    deps = [src, ORACLE / "m2_oracle.h"]
    if _stale(ORACLE_LIB, deps):
        _run(["gcc", "-O2", "-fopenmp", "-std=c11", "-shared", "-fPIC", str(src),
              "-o", str(ORACLE_LIB), "-lm"])
    if _stale(ORACLE_BIN, deps):
        _run(["gcc", "-O2", "-fopenmp", "-std=c11", "-DPGO_MAIN", str(src),
              "-o", str(ORACLE_BIN), "-lm"])
    return ORACLE_LIB


def build_reference() -> None:
    """Compile the reference itself from its own sources when they are present
    (validation only; outputs stay in oracle/_ref).  oracle/build_ref.sh finds
    the sources (PG_REFERENCE_DIR) and skips when they are absent."""
    outs = [ORACLE / "_ref" / name for name in ("combined_sieve", "combined_sieve_wheelfix", "gap_test_simple")]
    if all(o.exists() for o in outs):
        return
    subprocess.run(["bash", str(ORACLE / "build_ref.sh")], check=True, capture_output=True)


def build_arith_host() -> Path:
    """Host build of the device arithmetic header, for CPU unit tests."""
    BUILD.mkdir(parents=True, exist_ok=True)
    src = TESTS_NATIVE / "arith_host.cpp"
    if src.exists() and _stale(ARITH_HOST_LIB, [src] + _headers()):
        _run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", f"-I{CSRC}", str(src),
              "-o", str(ARITH_HOST_LIB)])
    return ARITH_HOST_LIB


def build_tune_host() -> Path:
    """Host build of the tuning cache logic, for CPU unit tests."""
    BUILD.mkdir(parents=True, exist_ok=True)
    src = TESTS_NATIVE / "tune_host.cpp"
    if src.exists() and _stale(TUNE_HOST_LIB, [src] + _headers()):
        _run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", f"-I{CSRC}", f"-I{INCLUDE}", str(src),
              "-o", str(TUNE_HOST_LIB)])
    return TUNE_HOST_LIB


def build_all(jobs: int = 8, verbose: bool = False, reference: bool = True) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_lib, jobs, verbose), ex.submit(build_oracle),
                ex.submit(build_arith_host), ex.submit(build_tune_host)]
        if reference:
            futs.append(ex.submit(build_reference))
        for f in futs:
            f.result()


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)
    shutil.rmtree(ORACLE_BUILD, ignore_errors=True)


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--lib", action="store_true")
    ap.add_argument("--clean", action="store_true")
    ap.add_argument("-j", type=int, default=8)
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args(argv)
    if a.clean:
        clean()
    if a.lib:
        build_lib(a.j, a.v)
    else:
        build_all(a.j, a.v)
    return 0


if __name__ == "__main__":
    sys.exit(main())
