"""Replica routing across ranks, run as two gloo processes on the CPU.

Every rank computes the scene owner map by itself and must agree with the others; the request
split must cover the stream exactly once; the merged latency percentiles must equal the
percentiles of the pooled latencies, and throughput uses the global first arrival and last
completion. Rank failure: a rank that raises before the gather makes the gather fail on the
other rank within the process-group timeout instead of hanging.
"""
from __future__ import annotations

import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from raytrace_gb300 import replicas  # noqa: E402


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def scene_sizes(n=64, seed=4):
    rng = np.random.default_rng(seed)
    return [int(x) for x in np.exp(rng.uniform(np.log(1e5), np.log(5e7), n))]


def request_stream(n=400, n_scenes=64, seed=5):
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(n_scenes)), float(t)) for t in np.cumsum(rng.exponential(1 / 200.0, n))]


def fake_serve(rank: int, reqs: list) -> replicas.RankResult:
    """Stand-in for a GPU server: latency and rays are pure functions of the request."""
    lat = np.array([1.0 + (s * 37 + int(t * 1000)) % 13 for s, t in reqs], np.float64)
    rays = sum(1000 + 17 * s for s, _ in reqs)
    t_first = min((t for _, t in reqs), default=0.0)
    t_last = max((t + l / 1e3 for (_, t), l in zip(reqs, lat)), default=0.0)
    return replicas.RankResult(rank, lat, rays, 256 * len(reqs), len(reqs), len(reqs), 0, t_first, t_last)


def worker(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        owner = replicas.owner_map(scene_sizes(), world)
        owners = [None] * world
        dist.all_gather_object(owners, owner)
        mine = replicas.split_requests(request_stream(), owner, world)[rank]
        ids = [None] * world
        dist.all_gather_object(ids, [(s, t) for s, t in mine])
        merged = replicas.gather(fake_serve(rank, mine))
        if rank == 0:
            q.put({"owners": owners, "ids": ids, "merged": merged})
    finally:
        dist.destroy_process_group()


def test_two_ranks_route_and_merge():
    world, port = 2, free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    owners, ids, merged = out["owners"], out["ids"], out["merged"]
    assert owners[0] == owners[1]                                  # agreed without talking
    stream = request_stream()
    got = sorted(x for part in ids for x in part)
    assert got == sorted(stream)                                   # every request exactly once
    for r, part in enumerate(ids):
        assert all(owners[0][s] == r for s, _ in part)
    # the merged figures equal a single-process computation over the whole stream
    whole = replicas.merge([fake_serve(0, stream)])
    for k in ("requests", "completed", "pixels", "rays", "p50_ms", "p99_ms", "max_ms"):
        assert merged[k] == whole[k], k
    assert merged["wall_s"] == pytest.approx(whole["wall_s"])


def test_owner_map_balances_bytes():
    sizes = scene_sizes()
    for world in (1, 2, 4, 8):
        owner = replicas.owner_map(sizes, world)
        load = np.bincount(owner, weights=sizes, minlength=world)
        assert len(set(owner)) == min(world, len(sizes))
        assert load.max() - load.min() <= max(sizes)               # greedy bound
    with pytest.raises(ValueError):
        replicas.owner_map(sizes, 0)


def failing_worker(rank: int, world: int, port: int, q) -> None:
    import datetime

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=5))
    if rank == 1:
        raise SystemExit(3)   # this rank dies before the gather (host-side failure)
    try:
        replicas.gather(fake_serve(0, request_stream(10)))
        q.put("no error")
    except Exception as e:   # the peer is gone: the collective reports it
        q.put(type(e).__name__)


def test_a_lost_rank_is_reported_not_hung():
    world, port = 2, free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=failing_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
    assert res != "no error"
    assert procs[1].exitcode == 3
