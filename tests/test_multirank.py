"""The N > 1 path of bench.py on CPU: two gloo ranks, each sieving its own
block of m (no data exchange), the slowest rank's time by a MAX all-reduce.
The ranks' files, concatenated in rank order, must be the single-job file of
the whole range: rows depend on their m alone, which is what lets the path
shard with no collective on the data."""
from __future__ import annotations

import hashlib
import socket

import pytest

JOB = dict(p=503, d=210, mstart=1234567, minc=600, sieve_length=5000, max_prime=20_000_000)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    import torch
    import torch.distributed as dist

    import bench
    import pgo

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        job = bench._rank_job(JOB, rank)
        text = pgo.method2(job["p"], job["d"], job["mstart"], job["minc"], job["sieve_length"],
                           job["max_prime"], threads=2)
        slowest = bench._max_over_ranks(torch, dist, rank, float(10 + rank))
        blocks = [None] * world
        dist.all_gather_object(blocks, (job["mstart"], job["minc"], text))
        if rank == 0:  # only small values through the queue
            q.put((slowest, [(m, n) for m, n, _ in blocks],
                   hashlib.md5(b"".join(t for _, _, t in blocks)).hexdigest()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_m_and_concatenate_to_the_whole_range():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    import pgo

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        slowest, blocks, md5 = q.get(timeout=240)  # read before joining
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    assert slowest == 11.0
    (m0, n0), (m1, n1) = blocks
    assert (m0, n0) == (JOB["mstart"], JOB["minc"]) and m1 == m0 + n0 and n1 == n0
    whole = pgo.method2(JOB["p"], JOB["d"], JOB["mstart"], 2 * JOB["minc"], JOB["sieve_length"],
                        JOB["max_prime"], threads=4)
    assert md5 == hashlib.md5(whole).hexdigest()
