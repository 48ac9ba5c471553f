"""Headless renderer CLI: render a seeded benchmark scene and write the image, or serve a
Poisson stream of requests.

Replaces the reference's window + glDrawPixels blit (main.cpp:197-208) with files: a binary
PPM of the uint8 image (Color::put, bottom-up rows flipped to top-down for viewers) and
optionally a PFM of the float colour.

    python -m raytrace_gb300.cli --config 2 --width 960 --height 540 --out frame.ppm
    python -m raytrace_gb300.cli --serve 800 --seconds 5      # the config-4 request stream
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

from . import RT_BUILD_CLUSTER, RT_FLAG_PROFILE, RT_FLAG_REF_TILES, BatchTuning, Context, SceneHost, Server


def write_ppm(path: str, rgb8: np.ndarray) -> None:
    h, w, _ = rgb8.shape
    with open(path, "wb") as f:
        f.write(f"P6\n{w} {h}\n255\n".encode())
        f.write(np.ascontiguousarray(rgb8[::-1]).tobytes())


def write_pfm(path: str, rgb: np.ndarray) -> None:
    h, w, _ = rgb.shape
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode())   # little endian, rows bottom-up as stored
        f.write(np.ascontiguousarray(rgb, "<f4").tobytes())


def serve(rate: float, seconds: float, n_scenes: int, budget_gb: int, plain: bool, slots: int = 512) -> dict:
    """A seeded Poisson stream of `rate` requests/s for `seconds` over the first `n_scenes`
    config-4 scenes (orbit cameras, resolutions 256^2..1080p, 1 spp, depth 3) through one server;
    returns its latency and throughput figures."""
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        scenes = list(ex.map(lambda i: SceneHost.config(4, i), range(n_scenes)))
    with Context(0) as ctx:
        ctx.set_build(RT_BUILD_CLUSTER)
        with Server(ctx, budget_gb << 30, max_inflight=slots, plain=plain, keep_images=False) as srv:
            for sc in scenes:
                srv.add_scene(sc)
            st = srv.run_poisson(rate, seconds, seed=4)
    return {"serve": rate, "seconds": seconds, "scenes": n_scenes, "plain": plain, **st}


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--config", type=int, default=0, help="benchmark scene 0..4")
    ap.add_argument("--index", type=int, default=0, help="scene number inside configs 3 and 4")
    ap.add_argument("--width", type=int, default=0)
    ap.add_argument("--height", type=int, default=0)
    ap.add_argument("--spp", type=int, default=0)
    ap.add_argument("--level", type=int, default=-1)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--ref-tiles", action="store_true", help="only the reference's 64x64-tile region")
    ap.add_argument("--stack", type=int, default=-1, help="traversal stack entries in shared memory: 0 or 8")
    ap.add_argument("--chunk", type=int, default=-1, help="shadow rays light-major in chunks of this many hits")
    ap.add_argument("--out", default="")
    ap.add_argument("--pfm", default="")
    ap.add_argument("--serve", type=float, default=0.0,
                    help="serve a Poisson stream of this many requests/s over the config-4 scenes instead")
    ap.add_argument("--seconds", type=float, default=1.0, help="length of the served stream")
    ap.add_argument("--scenes", type=int, default=64, help="config-4 scenes resident in the server")
    ap.add_argument("--budget-gb", type=int, default=120, help="the server's HBM budget")
    ap.add_argument("--slots", type=int, default=512, help="frame slots (1080p each) of the server")
    ap.add_argument("--plain", action="store_true", help="serve one request at a time (the comparison path)")
    a = ap.parse_args(argv)
    if a.serve > 0:
        print(json.dumps(serve(a.serve, a.seconds, a.scenes, a.budget_gb, a.plain, a.slots)))
        return 0
    scene = SceneHost.config(a.config, a.index)
    spp, lvl, seed = scene.params
    cam = scene.desc.camera
    w, h = a.width or cam.width, a.height or cam.height
    if (w, h) != (cam.width, cam.height):
        scene = scene.with_camera(w, h)
    spp = a.spp or spp
    lvl = lvl if a.level < 0 else a.level
    with Context(0) as ctx:
        if a.stack >= 0 or a.chunk >= 0:
            t = ctx.tuning()
            if a.stack >= 0:
                t.stack = a.stack
            if a.chunk >= 0:
                t.shadow_chunk = a.chunk
            ctx.set_tuning(t)
        sid = ctx.upload(scene)
        fid = ctx.frame(w, h)
        flags = RT_FLAG_PROFILE | (RT_FLAG_REF_TILES if a.ref_tiles else 0)
        st = None
        for _ in range(max(1, a.repeat)):
            st = ctx.render(sid, fid, ctx.render_desc(w, h, spp, lvl, flags=flags, seed=seed))
        out = ctx.download(fid, w, h, planes=False)
        info = {"config": a.config, "width": w, "height": h, "spp": spp, "max_level": lvl,
                "build_ms": ctx.build_ms(sid), **st.as_dict()}
    if a.out:
        write_ppm(a.out, out["rgb8"])
    if a.pfm:
        write_pfm(a.pfm, out["rgb"])
    print(json.dumps(info))
    return 0


if __name__ == "__main__":
    sys.exit(main())
