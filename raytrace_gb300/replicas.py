"""Replicas across GPUs: one renderer (and one server) per GPU, requests routed by scene id.

The rendering path has no exchange step — pixels, frames, scenes and requests are independent
— so several GPUs run as replicas: each owns a subset of the scenes, keeps them resident,
serves the requests that name them, and only the statistics are gathered. This module is the
host side of that: a deterministic owner map (every rank computes the same one, no
communication), the split of a request stream, and the exact merge of per-rank results.
"""
from __future__ import annotations

import heapq
from dataclasses import dataclass

import numpy as np


def owner_map(scene_bytes: list[int], world: int) -> list[int]:
    """Rank owning each scene: largest scenes first, each to the rank holding the fewest bytes
    (ties to the lower rank). Deterministic, so all ranks agree without communicating."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(scene_bytes)), key=lambda i: (-int(scene_bytes[i]), i))
    load = [(0, r) for r in range(world)]
    heapq.heapify(load)
    owner = [0] * len(scene_bytes)
    for i in order:
        b, r = heapq.heappop(load)
        owner[i] = r
        heapq.heappush(load, (b + int(scene_bytes[i]), r))
    return owner


def split_requests(requests: list, owner: list[int], world: int, scene_of=lambda r: r[0]) -> list[list]:
    """Requests per rank, in arrival order, by the owner of the scene each one names."""
    out: list[list] = [[] for _ in range(world)]
    for r in requests:
        out[owner[scene_of(r)]].append(r)
    return out


@dataclass
class RankResult:
    """What one rank reports after serving its share."""
    rank: int
    latencies_ms: np.ndarray
    rays: int
    pixels: int
    completed: int
    requests: int
    rejected: int
    t_first: float     # first arrival, seconds on a clock shared by the ranks
    t_last: float      # last completion, same clock


def merge(results: list[RankResult]) -> dict:
    """Whole-job figures: latencies pooled before taking percentiles (exact, not averaged),
    throughput = all rays / (last completion anywhere - first arrival anywhere)."""
    lat = np.concatenate([np.asarray(r.latencies_ms, np.float64) for r in results]) if results else np.zeros(0)
    t0 = min((r.t_first for r in results), default=0.0)
    t1 = max((r.t_last for r in results), default=0.0)
    wall = max(t1 - t0, 0.0)
    rays = sum(int(r.rays) for r in results)

    def pct(p: float) -> float:
        if lat.size == 0:
            return 0.0
        k = int(np.ceil(p * lat.size))
        return float(np.sort(lat)[min(max(k, 1), lat.size) - 1])

    return {
        "ranks": len(results),
        "requests": sum(r.requests for r in results),
        "completed": sum(r.completed for r in results),
        "rejected": sum(r.rejected for r in results),
        "pixels": sum(r.pixels for r in results),
        "rays": rays,
        "wall_s": wall,
        "mrays_per_s": rays / wall / 1e6 if wall > 0 else 0.0,
        "p50_ms": pct(0.50),
        "p99_ms": pct(0.99),
        "max_ms": float(lat.max()) if lat.size else 0.0,
    }


def gather(result: RankResult, group=None) -> dict | None:
    """Gather every rank's result on rank 0 (torch.distributed, any backend) and merge there;
    other ranks get None."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    objs = [None] * world if rank == 0 else None
    dist.gather_object(result, objs, dst=0, group=group)
    return merge(objs) if rank == 0 else None
