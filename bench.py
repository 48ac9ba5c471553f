#!/usr/bin/env python3
"""Benchmark of the GB300 renderer for the RayTracer per-pixel loop.

Workload (per step): one 1920x1080 frame of config 2 — 4 samples per pixel with Philox-jittered
sub-pixel offsets, recursion depth 4 (levels 0..4), a 1024x1024-vertex fBm terrain
(2,093,058 triangles) plus 64 spheres (16 refractive, IOR 1.5) and 4 point lights. Metric:
Mrays/s = traced ray segments (primary + reflect + refract + shadow) per second.

  value   device time of the render with the scene resident in HBM (CUDA events)
  e2e     the C-ABI call rt_render_host from host buffers: scene upload from page-locked host
          memory, device LBVH build, render and download of the uint8 image, wall clock
  roofline, cpu_baseline, clocks, per-kernel times: see the keys of the JSON line

`--impl reference` times the CPU oracle (a restatement of the reference's own algorithm,
checked bit-for-bit against the reference compiled from its sources) on a seeded sample of
the same frame's 64x64 tiles, with every host core.

Multi-GPU (torchrun, one rank per GPU): each rank renders its own copy of the frame
(replicas; the path has no exchange step), value = all ranks' rays / slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, SPP, LEVEL, SEED = 1920, 1080, 4, 4, 2
METRIC = "Mrays/s at 1080p (config 2: 1920x1080, 4 spp, depth 4)"
WORKLOAD = ("config2: 1920x1080 full frame, 4 spp Philox jitter (seed 2), depth 4, 1024^2-vertex fBm terrain "
            "(2,093,058 tris) + 64 spheres (16 refractive), 4 point lights")
CPU_SAMPLE_TILES = 4          # tiles of the reference's 30x16-tile region per CPU-baseline sample
REF_STEP_TILES = 2            # tiles per step of the --impl reference arm


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (getattr(self, "out", "") or "").splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic() -> float | None:
    """DRAM bytes per launch of the shadow kernel on this workload, from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "shadow_config2_traffic.txt")
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def cpu_tiles(n: int, seed: int) -> list[int]:
    import numpy as np

    bw, bh = W // 64, H // 64
    return sorted(np.random.default_rng(seed).choice(bw * bh, size=n, replace=False).tolist())


def cpu_sample(scene, n_tiles: int, seed: int, threads: int) -> dict:
    """The CPU oracle on `n_tiles` seeded tiles of the reference's 64x64-tile region."""
    from oracle import port

    tiles = cpu_tiles(n_tiles, seed)
    r = port.render(scene, W, H, SPP, LEVEL, SEED, ref_tiles=True, threads=threads, check=False, tiles=tiles, block=8)
    rays = int(r["counts"].sum())
    return {"rays": rays, "seconds": r["seconds"], "tiles": tiles, "mrays": rays / r["seconds"] / 1e6}


def run_reference(args) -> None:
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import raytrace_gb300 as rt

    threads = os.cpu_count() or 1
    scene = rt.SceneHost.config(2)
    for i in range(args.warmup):
        cpu_sample(scene, REF_STEP_TILES, 1000 + i, threads)
    rays, secs = 0, 0.0
    for i in range(args.steps):
        s = cpu_sample(scene, REF_STEP_TILES, i, threads)
        rays += s["rays"]
        secs += s["seconds"]
    v = rays / secs / 1e6
    sample = (f"{REF_STEP_TILES} seeded 64x64 tiles per step (of 480 in the reference's 1920x1024 region), 4 spp, "
              f"depth 4; CPU oracle restating the reference algorithm (octant lists, brute-force leaves)")
    print(json.dumps({
        "metric": METRIC, "value": round(v, 4), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * secs / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded config-2 scene)",
        "impl": "reference", "config": {"workload": WORKLOAD, "sample": sample},
        "cpu_baseline": {"value": round(v, 4), "unit": "Mrays/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(v, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def run_gpu(args) -> None:
    import numpy as np
    import torch

    import raytrace_gb300 as rt

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    scene = rt.SceneHost.config(2)
    scene.pin()
    ctx = rt.Context(local)
    sid = ctx.upload(scene)
    fid = ctx.frame(W, H)
    rd = ctx.render_desc(W, H, SPP, LEVEL, flags=0, seed=SEED)

    # untimed passes: work counts (algorithmic bytes) and per-kernel device times
    cnt = ctx.render(sid, fid, ctx.render_desc(W, H, SPP, LEVEL, flags=rt.RT_FLAG_COUNT_WORK, seed=SEED))
    prof = ctx.render(sid, fid, ctx.render_desc(W, H, SPP, LEVEL, flags=rt.RT_FLAG_PROFILE, seed=SEED))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")   # 256 MB > L2

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        ctx.render(sid, fid, rd)

    barrier()
    ctx.synchronize()
    torch.cuda.synchronize()
    step_ms, rays = [], 0
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)            # evict L2 between steps (outside the per-step events)
            torch.cuda.synchronize()
            st = ctx.render(sid, fid, rd)
            step_ms.append(st.ms)
            rays += st.total_rays()
        ctx.synchronize()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    barrier()
    dev_s = sum(step_ms) / 1e3

    # end to end through the C ABI with host buffers
    rgb8 = np.empty((H, W, 3), np.uint8)
    e2e_rd = ctx.render_desc(W, H, SPP, LEVEL, seed=SEED)
    ctx.render_host(scene, e2e_rd, W, H, want_rgb=False, rgb8=rgb8)   # warm
    barrier()
    e2e_rays, t0 = 0, time.perf_counter()
    for _ in range(args.steps):
        _, _, st = ctx.render_host(scene, e2e_rd, W, H, want_rgb=False, rgb8=rgb8)
        e2e_rays += st.total_rays()
    e2e_s = time.perf_counter() - t0
    barrier()

    if world > 1:
        t = torch.tensor([dev_s, e2e_s, wall], dtype=torch.float64, device=f"cuda:{local}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        r = torch.tensor([rays, e2e_rays], dtype=torch.float64, device=f"cuda:{local}")
        torch.distributed.all_reduce(r, op=torch.distributed.ReduceOp.SUM)
        dev_s, e2e_s, wall = t.tolist()
        rays, e2e_rays = r.tolist()
    if rank != 0:
        torch.distributed.destroy_process_group()
        return

    # roofline of the dominant kernel: algorithmic bytes per launch / measured launch time
    km = dict(zip(rt.KERNEL_KINDS, prof.kernel_ms))
    kl = dict(zip(rt.KERNEL_KINDS, prof.kernel_launches))
    dominant = max(("extend", "shadow", "shade"), key=lambda k: km[k])
    shadow_items = cnt.rays_shadow / 4           # one work item per hit, 4 lights
    alg = {
        # per shadow ray (one thread per hit and light): the 80-B hit record and a 24-B
        # fixed-point accumulate, then 64 B per internal node visited (the two 32-B child
        # records of the pair), 36 B per triangle tested, 16 B per sphere tested
        "shadow": cnt.rays_shadow * (80 + 24) + 64 * cnt.shadow_nodes_visited + 36 * cnt.shadow_tris_tested
        + 16 * cnt.shadow_spheres_tested,
        # ray 48 B read, hit 20 B written, then the traversal as above
        "extend": (cnt.rays_primary + cnt.rays_secondary) * (48 + 20) + 64 * cnt.nodes_visited
        + 36 * cnt.tris_tested + 16 * cnt.spheres_tested,
        # ray 64 B + hit 20 B read, children 64 B and shadow record 80 B written, accumulate 24 B
        "shade": (cnt.rays_primary + cnt.rays_secondary) * (64 + 20 + 24) + cnt.rays_secondary * 64
        + shadow_items * 80,
    }
    per_launch_bytes = alg[dominant] / max(1, kl[dominant])
    per_launch_s = km[dominant] / 1e3 / max(1, kl[dominant])
    achieved = per_launch_bytes / per_launch_s / 1e9
    peak, peak_kind = measured_peaks()
    traffic = profiled_traffic() if dominant == "shadow" else None

    cpu = None
    if world == 1 and not args.skip_cpu:
        s = cpu_sample(scene, CPU_SAMPLE_TILES, 0, os.cpu_count() or 1)
        cpu = {"value": round(s["mrays"], 4), "unit": "Mrays/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{CPU_SAMPLE_TILES} seeded 64x64 tiles {s['tiles']} of the 1920x1024 reference region, 4 spp, "
                         f"depth 4: {s['rays']} rays in {s['seconds']:.2f} s; CPU oracle restating the reference "
                         f"algorithm (octant lists, brute-force leaves)"}

    launches_per_step = sum(prof.kernel_launches)
    value = rays / dev_s / 1e6
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * dev_s / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded config-2 scene, generated on the host)",
        "config": {"workload": WORKLOAD, "width": W, "height": H, "spp": SPP, "max_level": LEVEL,
                   "triangles": int(scene.desc.n_tris), "parallelism": f"replicas x{world}",
                   "l2": "256 MB buffer written between timed steps; scene inputs (BVH 134 MB + triangles) exceed L2",
                   "rays_per_frame": {"primary": cnt.rays_primary, "secondary": cnt.rays_secondary,
                                      "shadow": cnt.rays_shadow}},
        "e2e": {"value": round(e2e_rays / e2e_s / 1e6, 2), "unit": "Mrays/s",
                "h2d_bytes_per_step": scene.nbytes, "d2h_bytes_per_step": W * H * 3,
                "what": "rt_render_host: pinned scene upload + LBVH build + render + uint8 download, wall clock"},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                     "peak_source": peak_kind, "alg_bytes_per_launch": int(per_launch_bytes),
                     "launch_ms": round(per_launch_s * 1e3, 4)},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "kernel_ms_per_frame": {k: round(v, 4) for k, v in km.items()},
        "kernel_launches_per_frame": kl,
        "wall_s_timed": round(wall, 4),
        "bvh_build_ms": round(ctx.build_ms(sid), 3),
    }
    print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU-baseline sample")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
