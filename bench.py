#!/usr/bin/env python
"""Throughput of the GB300 method2 sieve (and of the CPU reference arm).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload config2|config1|config3|batch64|served|ingest|prp]

One step = one whole method2 job (prime sieve, K mod p, large-prime marks,
small-prime rows, compaction, text) on the default workload: P=1511, d=2190,
minc=100000, SL=20000, max_prime=2e9, mstart=12345679 (a fixed draw inside
[1e6, 1e8) so the output can be checked against the reference's md5).
Headline metric: (m, p) pairs resolved per second = valid m x sieving primes
per second, whole job; primes/s is reported beside it.

`value` is device time (CUDA events on the library's stream) with the job's
tables resident; `e2e` is the public C-ABI call pgs_method2 with host output
(tables uploaded and the unknowns text copied back every step).  For N > 1
each rank sieves its own block of m (no data exchange; weak scaling).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "prime-gap_gb300"
for _p in (ROOT, PKG, ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

WORKLOADS = {
    "config1": dict(p=503, d=210, mstart=1234567, minc=10000, sieve_length=5000, max_prime=100_000_000),
    "config2": dict(p=1511, d=2190, mstart=12345679, minc=100000, sieve_length=20000,
                    max_prime=2_000_000_000),
    "config3": dict(p=3001, d=2190, mstart=123457, minc=100000, sieve_length=40000,
                    max_prime=10_000_000_000),
}
GOLDEN = ROOT / "tests" / "golden" / "goldens.json"
MIX_GOLDEN = ROOT / "tests" / "golden" / "mix_goldens.json"
PROFILE_TRAFFIC = ROOT / "profiles" / "large_kernel_traffic.txt"


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        rows = [r.split(", ") for r in Path(self.tmp.name).read_text().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _hbm_peak() -> tuple[float, str]:
    """Measured HBM copy bandwidth (GB/s) of the GB300s, or the
    fallback figure when the measurement file is absent."""
    f = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(f.read_text())["hbm_gbs"]), "of measured (MEASURED_PEAKS.json hbm_gbs, copy)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "of fallback (6.8 TB/s)"


def _traffic_per_launch() -> float | None:
    if not PROFILE_TRAFFIC.exists():
        return None
    for line in PROFILE_TRAFFIC.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch_config2:"):
            return float(line.split(":", 1)[1])
    return None


def _cpu_sample(job: dict, threads: int, rows_fraction: float = 1.0) -> dict:
    """The oracle port of the reference's method2 on the workload (the whole
    job by default; rows_fraction < 1 keeps only the first part of m, for
    warm-up): pairs/s on all host threads."""
    import pgo

    minc = max(1, int(job["minc"] * rows_fraction))
    pl = pgo.plan(job["p"], job["d"], job["mstart"], minc, job["sieve_length"], job["max_prime"])
    t = time.perf_counter()
    pgo.method2(job["p"], job["d"], job["mstart"], minc, job["sieve_length"], job["max_prime"],
                threads=threads)
    dt = time.perf_counter() - t
    primes = _count_primes(pl["prime_limit"])
    what = "whole job" if minc == job["minc"] else f"first {rows_fraction:.0%} of m (minc={minc})"
    return {"seconds": dt, "pairs": pl["valid_ms"] * primes, "primes": primes,
            "sample": f"{job}: {what}"}


def _percentiles(ms: list[float]) -> dict:
    """p50/p99 (nearest rank) of per-step times in ms."""
    v = sorted(ms)
    if not v:
        return {}
    rank = lambda q: v[min(len(v) - 1, max(0, int(round(q * len(v) + 0.5)) - 1))]
    return {"p50": rank(0.50), "p99": rank(0.99), "min": v[0], "max": v[-1], "n": len(v)}


_PI = {100_000_000: 5_761_455, 2_000_000_000: 98_222_287, 10_000_000_000: 455_052_511}


def _count_primes(limit: int) -> int:
    for k, v in _PI.items():
        if k - 1000 <= limit <= k:
            return v
    import pgo

    return len(pgo.primes(0, limit))


def run_reference(args, rank, world):
    """CPU reference arm: the oracle port of method2 on the host cores."""
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    if args.workload == "ingest":
        # the oracle's parse_unknown_line over the first 10% of config 2's m,
        # bitcompressed file written by the oracle itself
        import pgo

        j = dict(WORKLOADS["config2"])
        j["minc"] //= 10
        text = pgo.method2(j["p"], j["d"], j["mstart"], j["minc"], j["sieve_length"], j["max_prime"], 2,
                           threads=threads)
        secs, n = 0.0, 0
        for _ in range(max(1, args.steps)):
            t = time.perf_counter()
            lists = pgo.parse_unknowns(j["p"], j["d"], j["mstart"], j["minc"], j["sieve_length"],
                                       j["max_prime"], 2, text)
            secs += time.perf_counter() - t
            n += len(lists["dist"])
        value = n / secs
        line = {
            "impl": "reference", "metric": "unknowns ingested/s (parse_unknown_line replacement)",
            "value": value, "unit": "unknowns/s", "n_gpus": world, "steps": args.steps, "warmup": 0,
            "ms_per_step": secs / max(1, args.steps) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8/u32 integer", "data": "synthetic",
            "config": {"workload": "ingest", **j},
            "cpu_baseline": {"value": value, "unit": "unknowns/s", "cores": 1, "kind": "port",
                             "sample": f"bitcompressed file of {j}"},
            "e2e": {"value": value, "unit": "unknowns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return 0
    if args.workload == "prp":
        # the oracle's gap search over the first 64 m of config 2's unknowns
        # (lists from the oracle's own sieve), all host cores
        import pgo

        j = dict(WORKLOADS["config2"], minc=300)
        text = pgo.method2(j["p"], j["d"], j["mstart"], j["minc"], j["sieve_length"], j["max_prime"], 0,
                           threads=threads)
        lists = pgo.parse_unknowns(j["p"], j["d"], j["mstart"], j["minc"], j["sieve_length"], j["max_prime"], 0,
                                   text)
        secs, rows = 0.0, 0
        c = None
        for _ in range(max(1, args.steps)):
            c = _prp_cpu_sample(lists, j, threads)
            secs += c["seconds"]
            rows += c["rows"]
        value = rows / secs
        line = {
            "impl": "reference", "metric": "prime gaps searched/s (gap_test_gpu replacement)", "value": value,
            "unit": "m/s", "n_gpus": world, "steps": args.steps, "warmup": 0,
            "ms_per_step": secs / max(1, args.steps) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32 multi-precision", "data": "synthetic",
            "config": {"workload": "prp", **WORKLOADS["config2"], "min_merit": PRP_MIN_MERIT,
                       "one_side_skip": True},
            "cpu_baseline": {"value": value, "unit": "m/s", "cores": threads, "kind": "port",
                             "sample": c["sample"], "tests_per_s": c["tests_per_s"]},
            "e2e": {"value": value, "unit": "m/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return 0
    if args.workload in ("batch64", "served"):
        # every job of the 64-job mix, one after another on all host threads
        import workloads

        jobs = workloads.mixed_jobs(64, seed=4)
        _cpu_sample_jobs(jobs[:1], threads, 0.02)
        steps = []
        r = None
        for _ in range(max(1, args.steps)):
            r = _cpu_sample_jobs(jobs, threads)
            steps.append(r)
        secs = sum(x["seconds"] for x in steps)
        value = sum(x["pairs"] for x in steps) / secs
        r = dict(r, value=value)
        line = {
            "impl": "reference", "metric": "method2 sieve (m,p) pairs/s", "value": value,
            "unit": "pairs/s", "n_gpus": world, "steps": len(steps), "warmup": 1,
            "ms_per_step": secs / len(steps) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32/u64 integer", "data": "synthetic",
            "config": {"workload": args.workload, "jobs": len(jobs), "seed": 4},
            "same_config": True, "cpu_baseline": r,
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return 0
    job = WORKLOADS[args.workload]
    # warm-up: a 1% slice of m (loads the oracle and its threads); every
    # timed step is the whole job, the same config as the device arm
    for _ in range(args.warmup):
        _cpu_sample(job, threads, 0.01)
    secs, pairs, sample, per_step = 0.0, 0, "", []
    for _ in range(args.steps):
        r = _cpu_sample(job, threads)
        secs += r["seconds"]
        pairs += r["pairs"]
        sample = r["sample"]
        per_step.append(r["seconds"] * 1e3)
    value = pairs / secs
    line = {
        "impl": "reference", "metric": "method2 sieve (m,p) pairs/s", "value": value,
        "unit": "pairs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32/u64 integer", "data": "synthetic",
        "config": {"workload": args.workload, **job}, "same_config": True,
        "warmup_sample": "first 1% of m per warm-up step",
        "latency_ms": _percentiles(per_step),
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args, rank, world, local):
    import torch

    import pgsieve

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    job = _rank_job(WORKLOADS[args.workload], rank)
    spec = pgsieve.JobSpec(**job)
    sieve = pgsieve.Sieve(local)
    ext = torch.cuda.ExternalStream(sieve.stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    imad_peak = sieve.int_peak()

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    prep = sieve.prepare(spec)
    for _ in range(args.warmup):
        prep.run(True)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    stage_sum: dict[str, float] = {}
    step_ms = []
    barrier()
    clocks.start()
    for _ in range(args.steps):
        with torch.cuda.stream(ext):
            flush.zero_()  # > L2 (129 MB): every step starts cold
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            prep.run(True)
            e1.record(ext)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        st, _tot = prep.stage_ms()
        for k, v in st.items():
            stage_sum[k] = stage_sum.get(k, 0.0) + v
    barrier()
    clock_info = clocks.stop()
    total_ms = sum(step_ms)
    total_ms = _max_over_ranks(torch, dist, local, total_ms)

    stats: dict = {}
    data = prep.fetch(stats)
    prep.close()
    md5 = hashlib.md5(data).hexdigest()
    golden = json.loads(GOLDEN.read_text()).get(args.workload, {}) if GOLDEN.exists() else {}
    if golden and golden.get("max_prime") != spec.max_prime:
        golden = {}
    bit_exact = (md5 == golden["md5"]) if (golden and rank == 0) else None
    pairs_per_step = stats["rows"] * stats["primes"]
    value = pairs_per_step * world * args.steps / (total_ms * 1e-3)
    primes_per_s = stats["primes"] * world * args.steps / (total_ms * 1e-3)

    # end to end through the public call (tables up, text down, every step)
    for _ in range(min(args.warmup, 2)):
        sieve.method2_view(spec).close()
    barrier()
    e2e_s = []
    e2e_stats: dict = {}
    out_len = 0
    for _ in range(args.steps):
        t = time.perf_counter()
        view = sieve.method2_view(spec, e2e_stats)  # text is in host memory on return
        e2e_s.append(time.perf_counter() - t)
        out_len = len(view)
        view.close()
    barrier()
    e2e_total = _max_over_ranks(torch, dist, local, sum(e2e_s))
    plan = pgsieve.plan(spec)
    h2d = (4 * ((plan["k_bits"] + 31) // 32) + 4 * spec.minc + 4 * (2 * spec.sieve_length + 1)
           + 4 * plan["valid_ms"] + 2 * spec.sieve_length)
    e2e = {"value": pairs_per_step * world * args.steps / e2e_total, "unit": "pairs/s",
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(out_len + 64),
           "ms_per_step": e2e_total / args.steps * 1e3,
           "latency_ms": _percentiles([x * 1e3 for x in e2e_s])}

    # roofline of the dominant kernel (large-prime marks): integer-pipe bound.
    # Algorithmic integer ops per launch: 8 per continued-fraction level and
    # 6 per hit (large_kernel_model_ops).
    s1 = 4 * spec.sieve_length + 2
    n_windows = max(1, stats["prime_limit"] // (1 << 30) - (s1 + 1) // (1 << 30) + 1)
    large_ms = stage_sum.get("large", 0.0) / (args.steps * n_windows)
    model_ops = large_kernel_model_ops(spec, stats, plan) / n_windows
    achieved = model_ops / (large_ms * 1e-3) if large_ms else None
    # the measured traffic is config 2's (profiles/large_kernel_traffic.txt)
    traffic = (_traffic_per_launch() if args.workload == "config2"
               and spec.max_prime == WORKLOADS["config2"]["max_prime"] else None)
    roofline_int = {"kernel": "large_kernel<uint32_t>", "bound": "int", "achieved": achieved,
                    "peak": imad_peak, "unit": "int ops/s",
                    "frac": achieved / imad_peak if achieved else None, "traffic": traffic,
                    "peak_source": "measured live: IMAD microbenchmark (pgs_int_peak)",
                    "avg_launch_ms": large_ms}
    # the same kernel against HBM: its algorithmic bytes are the streamed
    # inputs, 12 B per prime (offset, walk step, start residue; the bitset of
    # hits stays in L2), against the measured copy bandwidth
    hbm_peak, hbm_src = _hbm_peak()
    alg_bytes = 12.0 * stats["primes"] / n_windows
    hbm_gbs = alg_bytes / (large_ms * 1e-3) / 1e9 if large_ms else None
    roofline = {"kernel": "large_kernel<uint32_t>", "bound": "hbm", "achieved": hbm_gbs, "peak": hbm_peak,
                "unit": "GB/s", "frac": hbm_gbs / hbm_peak if hbm_gbs else None, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": large_ms, "peak_source": hbm_src,
                "note": "integer-issue bound, not memory bound: see roofline_int"}

    if rank != 0:
        return 0
    cpu = None
    if world == 1 and not args.no_cpu:
        r = _cpu_sample(job, os.cpu_count() or 1)
        cpu = {"value": r["pairs"] / r["seconds"], "unit": "pairs/s", "cores": os.cpu_count(),
               "kind": "port", "sample": r["sample"], "seconds": round(r["seconds"], 2),
               "same_config": True}
    line = {
        "metric": "method2 sieve (m,p) pairs/s", "value": value, "unit": "pairs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32/u64 integer", "data": "synthetic",
        "config": {"workload": args.workload, **WORKLOADS[args.workload],
                   "l2": "flushed between steps (256 MiB write)", "parallelism": f"replicas x{world}"},
        "primes_per_s": primes_per_s, "bit_exact": bit_exact, "output_md5": md5,
        "latency_ms": _percentiles(step_ms),
        "stage_ms_per_step": {k: v / args.steps for k, v in stage_sum.items()},
        "e2e": e2e, "roofline": roofline, "roofline_int": roofline_int, "cpu_baseline": cpu,
        "clocks": clock_info,
        "gpu_launches": int(stats["launches"]) * args.steps,
    }
    print(json.dumps(line), flush=True)
    sieve.close()
    if dist:
        dist.destroy_process_group()
    return 0


def _pairs(res) -> int:
    return int(res.rows) * int(res.primes)


def _many_setup(args, rank, world, local):
    import torch

    import pgsieve
    import workloads

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    sieve = pgsieve.Sieve(local)
    t = time.perf_counter()
    sieve.reserve_table(4_000_000_000)  # the resident table every job draws from
    table_s = time.perf_counter() - t
    jobs = workloads.mixed_jobs(64, seed=4 + rank)  # each rank its own jobs
    return torch, pgsieve, workloads, dist, sieve, jobs, table_s


def _max_over_ranks(torch, dist, local, v: float) -> float:
    """The largest v over the ranks (the slowest rank's time)."""
    if not dist:
        return v
    dev = f"cuda:{local}" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _rank_job(job: dict, rank: int) -> dict:
    """Each rank sieves its own block of m, [mstart + rank*minc, mstart +
    (rank+1)*minc): rows depend on their m alone, so the blocks need no
    exchange and the ranks' files concatenate to the whole range's file."""
    return dict(job, mstart=job["mstart"] + rank * job["minc"])


def _cpu_sample_jobs(jobs, threads: int, rows_fraction: float = 1.0) -> dict:
    """The oracle on each of `jobs` in turn (whole jobs by default)."""
    secs, pairs, parts = 0.0, 0, []
    for j in jobs:
        r = _cpu_sample(dict(p=j.p, d=j.d, mstart=j.mstart, minc=j.minc, sieve_length=j.sieve_length,
                             max_prime=j.max_prime), threads, rows_fraction)
        secs += r["seconds"]
        pairs += r["pairs"]
        parts.append(f"P={j.p} d={j.d} minc={max(1, int(j.minc * rows_fraction))} SL={j.sieve_length} "
                     f"max_prime={j.max_prime}")
    what = "whole jobs" if rows_fraction >= 1 else f"first {rows_fraction:.0%} of the m"
    return {"value": pairs / secs, "unit": "pairs/s", "cores": threads, "kind": "port", "pairs": pairs,
            "sample": f"{what} of {len(jobs)} mix jobs" + (": " + "; ".join(parts) if len(parts) <= 4 else ""),
            "seconds": round(secs, 2)}


def _mix_reference_md5(jobs) -> dict:
    """Reference md5 of each job of the seed-4 mix (tests/golden/mix_goldens.json),
    keyed by job index; jobs whose parameters differ are left out."""
    if not MIX_GOLDEN.exists():
        return {}
    g = json.loads(MIX_GOLDEN.read_text())
    out = {}
    for i, j in enumerate(jobs):
        e = g.get(f"mix64_{i:02d}")
        if e and (e["p"], e["d"], e["mstart"], e["minc"], e["sieve_length"], e["max_prime"]) == (
                j.p, j.d, j.mstart, j.minc, j.sieve_length, j.max_prime):
            out[i] = e["md5"]
    return out


def run_batch(args, rank, world, local):
    """64 mixed jobs: the batched path (one CUDA graph over 8 streams, shared
    prime table) beside the plain path (each job alone, its own primes)."""
    torch, pgsieve, workloads, dist, sieve, jobs, table_s = _many_setup(args, rank, world, local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    # plain: every job through pgs_prepare/pgs_run, one after another
    preps = [sieve.prepare(j) for j in jobs]
    for p in preps:
        p.run(False)
    barrier()
    ext = torch.cuda.ExternalStream(sieve.stream)
    plain_ms = 0.0
    plain_steps = max(1, min(args.steps, 2))
    for _ in range(plain_steps):
        with torch.cuda.stream(ext):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            for p in preps:
                p.run(False)
            e1.record(ext)
        e1.synchronize()
        plain_ms += e0.elapsed_time(e1)
    # the plain path's stages summed over the jobs (one more pass, timed per stage)
    plain_stages: dict[str, float] = {}
    for p in preps:
        p.run(True)
        st, _ = p.stage_ms()
        for k, v in st.items():
            plain_stages[k] = plain_stages.get(k, 0.0) + v
    plain_md5 = []
    for p in preps:
        plain_md5.append(hashlib.md5(p.fetch()).hexdigest())
        p.close()
    plain_ms = _max_over_ranks(torch, dist, local, plain_ms) / plain_steps

    # batched: graph replay over the lanes
    batch = sieve.batch(jobs, lanes=args.lanes)
    for _ in range(args.warmup):
        batch.run(graph=True)
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    step_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        step_ms.append(batch.run(graph=True))
    barrier()
    clock_info = clocks.stop()
    total_ms = _max_over_ranks(torch, dist, local, sum(step_ms))
    pairs = 0
    bit_exact = True
    batch_md5 = []
    for i in range(len(jobs)):
        with batch.fetch_view(i) as v:
            pairs += _pairs(v.res)
            batch_md5.append(hashlib.md5(v.bytes()).hexdigest())
            bit_exact &= batch_md5[-1] == plain_md5[i]
    batch.close()
    ref_md5 = _mix_reference_md5(jobs)
    vs_ref = ({"checked": len(ref_md5), "equal": sum(batch_md5[i] == m for i, m in ref_md5.items())}
              if ref_md5 else None)
    value = pairs * world * args.steps / (total_ms * 1e-3)

    # end to end: pgs_method2_batch (tables up, every text down) per step
    for v in sieve.method2_batch_views(jobs):  # warm the pinned-buffer pool
        v.close()
    barrier()
    e2e_s = 0.0
    out_bytes = 0
    for _ in range(args.steps):
        t = time.perf_counter()
        views = sieve.method2_batch_views(jobs)  # every text is in host memory on return
        e2e_s += time.perf_counter() - t
        out_bytes = sum(len(v) for v in views)
        for v in views:
            v.close()
    e2e_s = _max_over_ranks(torch, dist, local, e2e_s)
    h2d = 0
    for j in jobs:
        pl = pgsieve.plan(j)
        h2d += (4 * ((pl["k_bits"] + 31) // 32) + 4 * j.minc + 4 * (2 * j.sieve_length + 1)
                + 4 * pl["valid_ms"] + 2 * j.sieve_length)
    if rank != 0:
        return 0
    cpu = None
    if world == 1 and not args.no_cpu:
        cpu = _cpu_sample_jobs(jobs[:3], os.cpu_count() or 1)
    line = {
        "metric": "method2 sieve (m,p) pairs/s", "value": value, "unit": "pairs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32/u64 integer", "data": "synthetic",
        "config": {"workload": "batch64", "jobs": len(jobs), "seed": 4, "lanes": args.lanes,
                   "mix": "P {503..3001}, d {1,210,2190,30030}, minc log-uniform 1e3..1e5, "
                          "SL 5000..40000, max_prime log-uniform 1e8..4e9",
                   "l2": "flushed between steps (256 MiB write); prime table 760 MB > L2",
                   "parallelism": f"replicas x{world}"},
        "plain_ms_per_batch": plain_ms, "plain_pairs_per_s": pairs * world / (plain_ms * 1e-3),
        "plain_stage_ms_sum": plain_stages,
        "batched_vs_plain": plain_ms / (total_ms / args.steps),
        "latency_ms": _percentiles(step_ms),
        "table_setup_s": table_s, "bit_exact_vs_plain": bit_exact, "bit_exact_vs_reference": vs_ref,
        "e2e": {"value": pairs * world * args.steps / e2e_s, "unit": "pairs/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(out_bytes),
                "ms_per_step": e2e_s / args.steps * 1e3},
        "cpu_baseline": cpu, "clocks": clock_info,
    }
    print(json.dumps(line), flush=True)
    sieve.close()
    if dist:
        dist.destroy_process_group()
    return 0


def run_ingest(args, rank, world, local):
    """The next consumer's ingestion (gap_stats' parse_unknown_line): config 2's
    unknowns as per-m lists, parsed on the device from each file format (host
    text in, host lists out) and read straight off the device after a run,
    beside the oracle's restatement of the parse on the host."""
    import ctypes

    import torch

    import pgo
    import pgsieve

    torch.cuda.set_device(local)
    job = dict(WORKLOADS["config2"])
    sieve = pgsieve.Sieve(local)
    lib = sieve.lib
    out = {}
    unknowns = 0
    for comp, name in ((0, "plain"), (1, "rle"), (2, "bitcompressed")):
        spec = pgsieve.JobSpec(**job, compression=comp)
        text = sieve.method2(spec)
        u = pgsieve.Unknowns()

        def parse():
            rc = lib.pgs_parse_unknowns(sieve.h, ctypes.byref(spec.c()), text, len(text), ctypes.byref(u))
            if rc != 0:
                raise pgsieve.PgsError(rc, lib.pgs_last_error(sieve.h).decode())
            n = u.total
            lib.pgs_unknowns_free(ctypes.byref(u))
            return n

        for _ in range(args.warmup):
            unknowns = parse()
        t = time.perf_counter()
        for _ in range(args.steps):
            parse()
        dt = (time.perf_counter() - t) / args.steps
        out[name] = {"ms": dt * 1e3, "text_bytes": len(text), "text_gb_per_s": len(text) / dt / 1e9,
                     "unknowns_per_s": unknowns / dt}
    # straight off the device after a run (no text)
    spec0 = pgsieve.JobSpec(**job)
    with sieve.prepare(spec0) as prep:
        prep.run(False)
        u = pgsieve.Unknowns()
        for _ in range(args.warmup):
            lib.pgs_fetch_unknowns(sieve.h, prep.h, ctypes.byref(u))
            lib.pgs_unknowns_free(ctypes.byref(u))
        t = time.perf_counter()
        for _ in range(args.steps):
            lib.pgs_fetch_unknowns(sieve.h, prep.h, ctypes.byref(u))
            lib.pgs_unknowns_free(ctypes.byref(u))
        dt = (time.perf_counter() - t) / args.steps
        out["device_lists"] = {"ms": dt * 1e3, "unknowns_per_s": unknowns / dt}
    # host parse of the same bytes by the oracle (single thread), on the
    # bitcompressed file of the first 10% of m
    cpu = None
    if not args.no_cpu:
        small = dict(job, minc=job["minc"] // 10)
        stext = sieve.method2(pgsieve.JobSpec(**small, compression=2))
        t = time.perf_counter()
        lists = pgo.parse_unknowns(small["p"], small["d"], small["mstart"], small["minc"],
                                   small["sieve_length"], small["max_prime"], 2, stext)
        dt = time.perf_counter() - t
        cpu = {"value": len(lists["dist"]) / dt, "unit": "unknowns/s", "cores": 1, "kind": "port",
               "sample": f"bitcompressed file of {small} ({len(stext)} bytes)", "seconds": round(dt, 3)}
    sieve.close()
    value = out["bitcompressed"]["unknowns_per_s"]
    line = {
        "metric": "unknowns ingested/s (parse_unknown_line replacement)", "value": value,
        "unit": "unknowns/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": out["bitcompressed"]["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8/u32 integer", "data": "synthetic",
        "config": {"workload": "ingest", **job, "unknowns": unknowns,
                   "value_is": "bitcompressed text on the host to lists on the host"},
        "formats": out, "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": "unknowns/s", "h2d_bytes_per_step": out["bitcompressed"]["text_bytes"],
                "d2h_bytes_per_step": 26301 * 24 + 4 * unknowns},
    }
    print(json.dumps(line), flush=True)
    return 0


PRP_MIN_MERIT = 18.0  # gap_test's default --min-merit (gap_common.h:49)
PRP_SAMPLE_ROWS = 64  # rows of the all-core reference arm (16 for the one-core baseline)


def _prp_rows_oracle(payload):
    """One worker of the CPU gap search: the oracle over a chunk of rows."""
    import prp_oracle as po

    p, d, sl, lists = payload
    k = po.primorial_k(p, d)
    res = po.gap_search(k, sl, lists, min_merit=PRP_MIN_MERIT, one_side_skip=True)
    return len(res), sum(r[2] + r[3] for r in res)


def _prp_cpu_sample(lists: dict, job: dict, workers: int, rows: int = PRP_SAMPLE_ROWS) -> dict:
    """The oracle's gap search (gap_test_gpu semantics) over the first `rows`
    rows on `workers` processes (spawned)."""
    import concurrent.futures
    import multiprocessing

    rows = min(rows, len(lists["m"]))
    chunks = []
    for w in range(workers):
        idx = list(range(w, rows, workers))
        if idx:
            chunks.append((job["p"], job["d"], job["sieve_length"],
                           {"m": [int(lists["m"][i]) for i in idx], "start": [int(lists["start"][i]) for i in idx],
                            "n_prev": [int(lists["n_prev"][i]) for i in idx],
                            "n_next": [int(lists["n_next"][i]) for i in idx], "dist": lists["dist"]}))
    t = time.perf_counter()
    if workers == 1:
        done = [_prp_rows_oracle(c) for c in chunks]
    else:
        ctx = multiprocessing.get_context("spawn")
        with concurrent.futures.ProcessPoolExecutor(max_workers=len(chunks), mp_context=ctx) as ex:
            done = list(ex.map(_prp_rows_oracle, chunks))
    dt = time.perf_counter() - t
    n_rows = sum(a for a, _ in done)
    tests = sum(b for _, b in done)
    return {"seconds": dt, "rows": n_rows, "tests": tests, "value": n_rows / dt, "tests_per_s": tests / dt,
            "sample": f"first {n_rows} m of config 2's unknowns, one-side skip, min_merit {PRP_MIN_MERIT}"}


def _prp_lists(sieve, job):
    import pgsieve

    with sieve.prepare(pgsieve.JobSpec(**job)) as prep:
        prep.run(False)
        return prep.unknowns()


def run_prp(args, rank, world, local):
    """The prime-gap search after the sieve (gap_test_gpu): config 2's unknown
    lists (26,301 m) from the host to the device, each side tested nearest
    first with the base-2 strong probable-prime test until a probable prime,
    gap_test_gpu's one-side skip at min_merit 18, results back to the host."""
    import torch
    import pgsieve

    torch.cuda.set_device(local)
    job = dict(WORKLOADS["config2"])
    sieve = pgsieve.Sieve(local)
    lists = _prp_lists(sieve, job)
    rows = len(lists["m"])

    def step():
        return sieve.prp_gaps(job["p"], job["d"], job["sieve_length"], lists, min_merit=PRP_MIN_MERIT,
                              one_side_skip=True)

    for _ in range(args.warmup):
        res, st = step()
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    t = time.perf_counter()
    launched = counted = rounds = 0
    for _ in range(args.steps):
        res, st = step()
        launched += st["prp_tests"]
        rounds += st["rounds"]
        counted += sum(r[2] + r[3] for r in res)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t) / args.steps
    clock_info = clocks.stop()
    # the same search over a prepared job's lists in place (no host round trip)
    with sieve.prepare(pgsieve.JobSpec(**job)) as prep:
        prep.run(False)
        prep.prp_gaps(min_merit=PRP_MIN_MERIT, one_side_skip=True)
        t = time.perf_counter()
        for _ in range(2):
            prep.prp_gaps(min_merit=PRP_MIN_MERIT, one_side_skip=True)
        prepared_ms = (time.perf_counter() - t) / 2 * 1e3
    peak = sieve.int_peak()
    # roofline: Montgomery products of n limbs, 2n^2 32-bit multiply-adds
    # (64-bit results: two IMAD issue slots each) per product, one product per
    # bit of N, over every test launched
    import prp_oracle as po

    n = st["limbs"]
    bits = po.primorial_k(job["p"], job["d"]).bit_length() + int(max(lists["m"])).bit_length()
    ops = launched / args.steps * bits * 2 * n * n * 2
    cpu = None
    if not args.no_cpu:
        c = _prp_cpu_sample(lists, job, 1, rows=16)
        cpu = {"value": c["value"], "unit": "m/s", "cores": 1, "kind": "port", "sample": c["sample"],
               "tests_per_s": c["tests_per_s"], "seconds": round(c["seconds"], 2)}
    sieve.close()
    value = rows / dt
    line = {
        "metric": "prime gaps searched/s (gap_test_gpu replacement)", "value": value, "unit": "m/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 multi-precision",
        "data": "synthetic",
        "config": {"workload": "prp", **job, "rows": rows, "unknowns": int(len(lists["dist"])),
                   "min_merit": PRP_MIN_MERIT, "one_side_skip": True, "bits": bits,
                   "value_is": "lists on the host to gaps on the host"},
        "prp_tests_per_s": counted / args.steps / dt, "prp_launched_per_s": launched / args.steps / dt,
        "rounds_per_step": rounds / args.steps, "from_prepared_job_ms": prepared_ms,
        "roofline": {"kernel": f"prp_kernel<{n // 8}>", "bound": "int", "achieved": ops / dt, "peak": peak,
                     "unit": "int ops/s", "frac": ops / dt / peak, "traffic": None,
                     "peak_source": "measured live: IMAD microbenchmark (pgs_int_peak)"},
        "cpu_baseline": cpu, "clocks": clock_info, "gpu_launches": args.steps * (2 + 3 * rounds // args.steps),
        "e2e": {"value": value, "unit": "m/s", "h2d_bytes_per_step": rows * 24 + 4 * int(len(lists["dist"])),
                "d2h_bytes_per_step": rows * 20},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_served(args, rank, world, local):
    """1000 mixed requests, Poisson arrivals at 80% of the batched job rate,
    admitted against a 150 GB device budget; p50/p99 latency."""
    torch, pgsieve, workloads, dist, sieve, jobs64, table_s = _many_setup(args, rank, world, local)
    import random

    with sieve.batch(jobs64, lanes=args.lanes) as b:
        b.run(graph=True)
        rate = 0.8 * len(jobs64) / (b.run(graph=True) * 1e-3)
    rng = random.Random(1000 + rank)
    jobs = [workloads.mixed_job(rng) for _ in range(args.requests)]
    arrivals = workloads.poisson_arrivals(len(jobs), rate, seed=7 + rank)
    import concurrent.futures
    import zlib

    # CRC-32 and length of every output (zlib releases the GIL and reads the
    # pinned result in place); four threads, so the server's own host threads
    # keep their cores
    hasher = concurrent.futures.ThreadPoolExecutor(max_workers=4)

    def md5_close(v):
        try:
            return (zlib.crc32(v.view), len(v))
        finally:
            v.close()

    # every request's result alone on the plain path, hashed off the main thread
    want_f = [hasher.submit(md5_close, sieve.method2_view(j)) for j in jobs]
    want = [f.result() for f in want_f]
    got_f = [None] * len(jobs)
    pairs = 0
    barrier_t = torch.cuda.synchronize
    barrier_t()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    with sieve.server(hbm_budget=150 << 30, lanes=args.lanes) as srv:
        tickets = [None] * len(jobs)
        clocks.start()
        t0 = time.perf_counter()

        def submitter():
            for i, (j, ta) in enumerate(zip(jobs, arrivals)):
                dt = t0 + ta - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                tickets[i] = srv.submit(j)

        th = threading.Thread(target=submitter)
        th.start()
        lat = []
        for i in range(len(jobs)):
            while tickets[i] is None:
                time.sleep(0.0002)
            v, ms = srv.wait_view(tickets[i], timeout_ms=600_000)
            pairs += _pairs(v.res)
            got_f[i] = hasher.submit(md5_close, v)  # hashed and freed by the pool
            lat.append(ms)
        th.join()
        wall = time.perf_counter() - t0
        st = srv.stats()
        clock_info = clocks.stop()
    wall = _max_over_ranks(torch, dist, local, wall)
    got = [f.result() for f in got_f]
    hasher.shutdown()
    if rank != 0:
        return 0
    lat.sort()
    line = {
        "metric": "method2 sieve (m,p) pairs/s", "value": pairs * world / wall, "unit": "pairs/s",
        "n_gpus": world, "steps": 1, "warmup": args.warmup, "ms_per_step": wall * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32/u64 integer", "data": "synthetic",
        "config": {"workload": "served", "requests": len(jobs), "arrival_rate_per_s": rate,
                   "hbm_budget_bytes": 150 << 30, "lanes": args.lanes,
                   "parallelism": f"replicas x{world}"},
        "jobs_per_s": len(jobs) * world / wall,
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
                       "mean": sum(lat) / len(lat), "max": lat[-1]},
        "server": st, "bit_exact_vs_plain": {"checked": len(jobs), "by": "crc32 and length of every output",
                                             "equal": sum(g == w for g, w in zip(got, want))},
        "bit_exact_all": got == want,
        "table_setup_s": table_s, "clocks": clock_info,
        "e2e": {"value": pairs * world / wall, "unit": "pairs/s", "h2d_bytes_per_step": None,
                "d2h_bytes_per_step": None},
    }
    print(json.dumps(line), flush=True)
    sieve.close()
    if dist:
        dist.destroy_process_group()
    return 0


def run_tune(args, rank, world, local):
    """The autotuner: each job class of configs 1-3 and of the 64-job mix
    tuned on this device (pgs_tune: one knob at a time, median of 5 runs),
    then the mix batched with the default knobs and with the tuned ones."""
    import torch

    import pgsieve
    import workloads

    torch.cuda.set_device(local)
    table = []
    t0 = time.perf_counter()
    with pgsieve.Sieve(local, load_tuning=False) as s:
        for name in ("config1", "config2", "config3"):
            spec = pgsieve.JobSpec(**WORKLOADS[name])
            knobs, ms_def, ms_tuned = s.tune(spec, reps=5)
            table.append({"job": name, "class": pgsieve.tuning_class(spec), "knobs": knobs,
                          "ms_default": ms_def, "ms_tuned": ms_tuned})
        jobs = workloads.mixed_jobs(64, seed=4)
        seen = {r["class"] for r in table}  # a mix job of a config's class keeps the config's knobs
        for j in jobs:
            c = pgsieve.tuning_class(j)
            if c in seen:
                continue
            seen.add(c)
            knobs, ms_def, ms_tuned = s.tune(j, reps=5)
            table.append({"job": "mix64", "class": c, "knobs": knobs, "ms_default": ms_def,
                          "ms_tuned": ms_tuned})
        tune_s = time.perf_counter() - t0
        if args.tuning_out:
            s.tuning_save(args.tuning_out)
        s.reserve_table(4_000_000_000)
        with s.batch(jobs, lanes=args.lanes) as b:  # tuned knobs (this context's entries)
            for _ in range(args.warmup):
                b.run(graph=True)
            tuned = [b.run(graph=True) for _ in range(args.steps)]
            pairs = 0
            for i in range(len(jobs)):
                with b.fetch_view(i) as v:
                    pairs += _pairs(v.res)
    with pgsieve.Sieve(local, load_tuning=False) as s:
        s.reserve_table(4_000_000_000)
        with s.batch(jobs, lanes=args.lanes) as b:
            for _ in range(args.warmup):
                b.run(graph=True)
            default = [b.run(graph=True) for _ in range(args.steps)]
    mix = [r for r in table if r["job"] == "mix64"]
    line = {
        "metric": "method2 sieve (m,p) pairs/s", "value": pairs * args.steps / (sum(tuned) * 1e-3),
        "unit": "pairs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sum(tuned) / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32/u64 integer", "data": "synthetic",
        "config": {"workload": "tune", "value_is": "batch64 with tuned knobs"},
        "batch64_ms": {"default": _percentiles(default), "tuned": _percentiles(tuned)},
        "tuning_s": tune_s, "classes": len(table),
        "mix_sum_ms": {"default": sum(r["ms_default"] for r in mix), "tuned": sum(r["ms_tuned"] for r in mix)},
        "table": table,
    }
    print(json.dumps(line), flush=True)
    return 0


def large_kernel_model_ops(spec, stats, plan) -> float:
    """Model of the large-prime phase's integer work (ops per job).

    The parity-reduced walk visits minc*(2SL+1)/p / 4 hits per prime for d
    even (only odd m and even X) and / 2 for d odd; summed over the phase's
    primes with Mertens' estimate that is minc*(2SL+1)*(ln ln P1 - ln ln P0)/4.
    6 integer ops per hit, plus one continued fraction per prime at 8 ops per
    level over 0.843*ln(p/w) levels (Heilbronn's mean)."""
    import math

    w = 2 * spec.sieve_length + 1
    p0 = 4 * spec.sieve_length + 2
    p1 = stats["prime_limit"]
    reduce = 4 if spec.d % 2 == 0 else 2
    hits = spec.minc * w * (math.log(math.log(p1)) - math.log(math.log(p0))) / reduce
    nprimes = stats["primes"]
    levels = 0.843 * math.log(max(p1 / 2, p0) / (w / 2))
    return 6 * hits + 8 * levels * nprimes


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="config2",
                    choices=sorted(WORKLOADS) + ["batch64", "served", "ingest", "prp", "tune"])
    ap.add_argument("--lanes", type=int, default=8, help="streams of the batched/served paths")
    ap.add_argument("--requests", type=int, default=1000, help="served requests")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--tuning-out", default="", help="tune workload: write the tuning cache file here")
    ap.add_argument("--max-prime", type=int, default=0,
                    help="override the workload's max_prime (small profiling runs)")
    args = ap.parse_args()
    rank, world, local = _dist()
    if args.workload == "ingest" and args.impl == "gb300":
        return run_ingest(args, rank, world, local)
    if args.workload == "prp" and args.impl == "gb300":
        return run_prp(args, rank, world, local)
    if args.workload in ("batch64", "served") and args.impl == "gb300":
        return (run_batch if args.workload == "batch64" else run_served)(args, rank, world, local)
    if args.workload == "tune":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the tuner has no CPU counterpart"}))
            return 0
        return run_tune(args, rank, world, local)
    if args.max_prime:
        WORKLOADS[args.workload] = dict(WORKLOADS[args.workload], max_prime=args.max_prime)
        args.workload_note = "max_prime overridden"
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_gb300(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
