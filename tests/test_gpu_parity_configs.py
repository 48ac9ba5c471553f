"""GPU parity at the benchmark configurations' stated sizes, against the CPU oracle.

* config 0: the whole 512x512 frame, every pixel checked;
* config 2: the whole 1920x1080, 4-spp, depth-4 frame the benchmark times, rendered on the GPU;
  16 of its 64x64 tiles, one per tile row (the benchmark's CPU sample), rendered by the oracle;
* config 3: 8 scenes of the batched workload through rt_batch_render (shared waves, CUDA graph),
  three tiles of each frame against the oracle — not against the GPU's own plain path;
* config 4: 4 requests with orbit cameras through the continuous-batching server, three tiles
  of each image against the oracle rendering the same scene from the same camera.

The rule is the one of every parity test here: on each pixel the oracle does not mark
ambiguous, the primary hit object and primitive are the oracle's, the hit distance is the
oracle's bit for bit, and the colour before Color::put is within 1e-4 per channel (absolute).
Ambiguity is a brute-force pass over every primitive per ray, which costs seconds per pixel on
the 2.1M-triangle terrain, so it runs only on the pixels that differ; each test prints how
many pixels it compared, how many differ, and how many of those the oracle marks ambiguous
(run with -s)."""
from __future__ import annotations

import json

import numpy as np
import pytest

import raytrace_gb300 as rt
from bench import cpu_tiles
from oracle import port

pytestmark = pytest.mark.gpu
TOL = 1e-4


def tile_mask(tiles, w, h):
    m = np.zeros((h, w), bool)
    bw = w // 64
    for t in tiles:
        r, c = (t // bw) * 64, (t % bw) * 64
        m[r:r + 64, c:c + 64] = True
    return m


def strat_tiles(w, h, n, seed):
    """n distinct 64x64 tiles of the reference's tile region: the one at the frame's centre
    (where the scenes' meshes sit) and n - 1 more, one from each of n - 1 bands of tile rows."""
    bw, bh = w // 64, h // 64
    rng = np.random.default_rng(seed)
    tiles = {(bh // 2) * bw + bw // 2}
    for k in range(n - 1):
        lo, hi = (k * bh) // (n - 1), max((k * bh) // (n - 1) + 1, ((k + 1) * bh) // (n - 1))
        for _ in range(100):
            t = int(rng.integers(lo, hi)) * bw + int(rng.integers(bw))
            if t not in tiles:
                tiles.add(t)
                break
    return sorted(tiles)


def oracle_compare(scene, out, w, h, spp, lvl, seed, tiles, ids=True, label=""):
    """The GPU frame `out` against the oracle on `tiles`; returns and prints the counts."""
    ref = port.render(scene, w, h, spp, lvl, seed, ref_tiles=True, check=False, tiles=tiles, block=8)
    mask = tile_mask(tiles, w, h)
    d = np.abs(out["rgb"] - ref["rgb"]).max(axis=2)
    bad = mask & ~(d <= TOL)
    if ids:
        bad |= mask & ((out["obj"] != ref["obj"]) | (out["prim"] != ref["prim"]))
    amb = np.zeros_like(mask)
    if bad.any():
        bw = w // 64
        bad_tiles = sorted({(y // 64) * bw + x // 64 for y, x in zip(*np.nonzero(bad))})
        chk = port.render(scene, w, h, spp, lvl, seed, ref_tiles=True, check=True, tiles=bad_tiles, block=2,
                          check_pixels=bad)
        amb = chk["ambiguous"] & bad
        unexplained = bad & ~amb
        assert not unexplained.any(), (f"{label}: {int(unexplained.sum())} unambiguous pixels differ, e.g. "
                                       f"{list(zip(*np.nonzero(unexplained)))[:8]}")
    if ids:
        same = mask & (out["obj"] == ref["obj"]) & (out["prim"] == ref["prim"]) & (ref["obj"] >= 0)
        np.testing.assert_array_equal(out["t"][same].view(np.uint32), ref["t"][same].view(np.uint32))
    ok = mask & ~amb
    lsb = np.abs(out["rgb8"].astype(int) - ref["rgb8"].astype(int)).max(axis=2)
    assert lsb[ok].max(initial=0) <= 1, label
    stats = {"case": label, "pixels": int(mask.sum()), "hit_pixels": int((mask & (ref["obj"] >= 0)).sum()) if ids else None,
             "differing": int(bad.sum()), "ambiguous": int(amb.sum()),
             "max_rgb_diff_unambiguous": float(d[ok].max(initial=0.0)), "rays": int(ref["counts"].sum())}
    print("parity", json.dumps(stats))
    return stats


def test_config0_full_frame_matches_oracle(ctx):
    """Config 0 at its stated 512x512, the whole frame, every pixel checked for ambiguity."""
    scene = rt.SceneHost.config(0)
    w, h = 512, 512
    sid = ctx.upload(scene)
    fid = ctx.frame(w, h)
    try:
        ctx.render(sid, fid, ctx.render_desc(w, h, 1, 3, flags=rt.RT_FLAG_HIT_PLANES))
        out = ctx.download(fid, w, h)
    finally:
        ctx.release_frame(fid)
        ctx.release_scene(sid)
    ref = port.render(scene, w, h, 1, 3, 0, ref_tiles=False, check=True)
    a = ref["ambiguous"]
    ids_equal = (out["obj"] == ref["obj"]) & (out["prim"] == ref["prim"])
    assert not (~ids_equal & ~a).any()
    same = ids_equal & (ref["obj"] >= 0)
    np.testing.assert_array_equal(out["t"][same].view(np.uint32), ref["t"][same].view(np.uint32))
    d = np.abs(out["rgb"] - ref["rgb"]).max(axis=2)
    assert not (~(d <= TOL) & ~a).any(), float(d[~a].max())
    assert np.abs(out["rgb8"].astype(int) - ref["rgb8"].astype(int)).max(axis=2)[~a].max() <= 1
    print("parity", json.dumps({"case": "config0 512x512", "pixels": w * h, "ambiguous": int(a.sum()),
                                "differing": int((~ids_equal | ~(d <= TOL)).sum()),
                                "max_rgb_diff_unambiguous": float(d[~a].max())}))


def test_largest_dropin_frame_matches_oracle(ctx):
    """2048x2048, the largest frame the drop-in's output buffer holds (RayTracer.cpp:603): every
    pixel against the oracle."""
    w = h = 2048
    scene = rt.SceneHost.small(21, 10, 6, w, h, 3)
    sid = ctx.upload(scene)
    fid = ctx.frame(w, h)
    try:
        ctx.render(sid, fid, ctx.render_desc(w, h, 1, 3, flags=rt.RT_FLAG_HIT_PLANES))
        out = ctx.download(fid, w, h)
    finally:
        ctx.release_frame(fid)
        ctx.release_scene(sid)
    stats = oracle_compare(scene, out, w, h, 1, 3, 0, list(range((w // 64) * (h // 64))), label="2048x2048")
    assert stats["pixels"] == w * h


def test_config2_benchmark_frame_matches_oracle_on_row_stratified_tiles(ctx):
    """The frame bench.py times (1920x1080, 4 spp Philox jitter, depth 4, 2.1M-triangle terrain,
    64 spheres of which 16 refract, 4 lights), rendered whole on the GPU; 16 tiles, one per
    tile row of the reference's 30x16-tile region, against the oracle."""
    scene = rt.SceneHost.config(2)
    w, h, spp, lvl, seed = 1920, 1080, 4, 4, 2
    sid = ctx.upload(scene)
    fid = ctx.frame(w, h)
    try:
        ctx.render(sid, fid, ctx.render_desc(w, h, spp, lvl, flags=rt.RT_FLAG_HIT_PLANES, seed=seed))
        out = ctx.download(fid, w, h)
    finally:
        ctx.release_frame(fid)
        ctx.release_scene(sid)
    tiles = cpu_tiles(16, 0)
    assert len({t // (w // 64) for t in tiles}) == 16   # one per tile row
    s = oracle_compare(scene, out, w, h, spp, lvl, seed, tiles, label="config2 1920x1080 4spp depth4, 16 tiles")
    assert s["hit_pixels"] > 20000   # the sample covers the terrain, not only sky


CONFIG3_SCENES = [0, 1, 2, 4, 5, 6, 9, 11]   # 256^2 .. 1080p, 1,280 .. 264,500 triangles


def test_config3_batch_matches_oracle(ctx):
    """Eight config-3 scenes rendered together through rt_batch_render (shared waves, one CUDA
    graph per wave) with the hierarchy the benchmark uses for resident scenes; each frame's
    ids, distances and colours against the oracle on three of its tiles."""
    scenes = [rt.SceneHost.config(3, i) for i in CONFIG3_SCENES]
    sids, fids, rds, sizes = [], [], [], []
    ctx.set_build(rt.RT_BUILD_CLUSTER)
    try:
        for sc in scenes:
            c = sc.desc.camera
            sids.append(ctx.upload(sc))
            fids.append(ctx.frame(c.width, c.height))
            rds.append(ctx.render_desc(c.width, c.height, 1, 3, flags=rt.RT_FLAG_HIT_PLANES))
            sizes.append((c.width, c.height))
    finally:
        ctx.set_build(rt.RT_BUILD_RADIX)
    try:
        ctx.batch(sids, fids, rds)
        outs = [ctx.download(f, w, h) for f, (w, h) in zip(fids, sizes)]
    finally:
        for f in fids:
            ctx.release_frame(f)
        for s in sids:
            ctx.release_scene(s)
    total_hits = 0
    for i, sc, out, (w, h) in zip(CONFIG3_SCENES, scenes, outs, sizes):
        s = oracle_compare(sc, out, w, h, 1, 3, 0, strat_tiles(w, h, 3, i),
                           label=f"config3 scene {i} {w}x{h} {int(sc.desc.n_tris)} tris")
        total_hits += s["hit_pixels"]
    assert total_hits > 10000


CONFIG4_REQUESTS = [(49, 1920, 1080), (19, 1024, 768), (0, 512, 512), (2, 256, 256)]   # (scene, width, height)


def test_config4_served_requests_match_oracle(ctx):
    """Four requests with seeded orbit cameras (azimuth U[0,360), elevation U[10,60]) on
    config-4 scenes, admitted together into the continuous-batching server (their samples share
    waves); each image against the oracle rendering that scene from that camera on three tiles."""
    scenes = {i: rt.SceneHost.config(4, i) for i, _, _ in CONFIG4_REQUESTS}
    rng = np.random.default_rng(4)
    ctx.set_build(rt.RT_BUILD_CLUSTER)
    try:
        with rt.Server(ctx, 24 << 30, max_inflight=8, keep_images=True, queue_rays=1 << 22) as srv:
            ids = {i: srv.add_scene(sc) for i, sc in scenes.items()}
            reqs = []
            for i, w, h in CONFIG4_REQUESTS:
                cam = rt.orbit_camera(srv.camera(ids[i]), float(rng.uniform(0, 360)), float(rng.uniform(10, 60)), w, h)
                reqs.append((i, w, h, cam, srv.submit(ids[i], w, h, cam, 0)))
            srv.drain()
            st = srv.stats()
            results = [(i, w, h, cam, srv.result(rid)) for i, w, h, cam, rid in reqs]
    finally:
        ctx.set_build(rt.RT_BUILD_RADIX)
    assert st["completed"] == len(CONFIG4_REQUESTS)
    for i, w, h, cam, res in results:
        assert res["status"] == rt.RT_OK
        d = rt.SceneDesc.from_buffer_copy(scenes[i].desc)
        d.camera = cam
        view = rt.SceneHost.from_desc(d, 1, 3, 0)
        oracle_compare(view, {"rgb": res["rgb"], "rgb8": res["rgb8"]}, w, h, 1, 3, 0, strat_tiles(w, h, 3, 100 + i),
                       ids=False, label=f"config4 scene {i} {w}x{h} orbit camera")
