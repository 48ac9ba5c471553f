"""Batched and served rendering on the GPU.

* rt_batch_render: many (scene, frame) jobs in shared waves give, per frame, the very bits of
  the plain one-scene render (colours accumulate as exact fixed-point sums).
* rt_server: each request's image is the same alone, in a mix admitted while other requests
  are in flight, split over many waves, through the plain one-at-a-time mode, and after its
  scene was evicted and rebuilt under a small HBM budget; one request is checked against the
  CPU oracle. Errors (unknown scene, oversize request, budget) are reported, not hidden.
"""
from __future__ import annotations

import numpy as np
import pytest

import raytrace_gb300 as rt

pytestmark = pytest.mark.gpu


def small_scenes():
    # refractive spheres in two of them: those waves use the 2^level queue bound
    return [rt.SceneHost.small(seed=s, n_spheres=n, ico_freq=f, width=64, height=64, refractive_every=r)
            for s, n, f, r in [(21, 6, 6, 0), (22, 10, 3, 3), (23, 4, 10, 0), (24, 8, 0, 2)]]


def plain_render(ctx, scene, w, h, camera=None, spp=1, level=3, seed=0):
    sid = ctx.upload(scene)
    fid = ctx.frame(w, h)
    try:
        ctx.render(sid, fid, ctx.render_desc(w, h, spp, level, seed=seed, camera=camera))
        return ctx.download(fid, w, h, planes=False)
    finally:
        ctx.release_frame(fid)
        ctx.release_scene(sid)


def test_batch_equals_plain_renders(ctx):
    scenes = [rt.SceneHost.config(3, i) for i in range(6)] + small_scenes()
    sizes = [(96, 64), (128, 128), (80, 60), (200, 120), (64, 64), (160, 90), (72, 72), (128, 96), (96, 96),
             (100, 50)]
    sids, fids, rds = [], [], []
    for sc, (w, h) in zip(scenes, sizes):
        sids.append(ctx.upload(sc))
        fids.append(ctx.frame(w, h))
        rds.append(ctx.render_desc(w, h, 1, 3))
    try:
        ctx.batch(sids, fids, rds)
        for sc, sid, fid, (w, h) in zip(scenes, sids, fids, sizes):
            got = ctx.download(fid, w, h, planes=False)
            ref = plain_render(ctx, sc, w, h)
            assert np.array_equal(got["rgb"], ref["rgb"]), (w, h)
            assert np.array_equal(got["rgb8"], ref["rgb8"])
    finally:
        for f in fids:
            ctx.release_frame(f)
        for s in sids:
            ctx.release_scene(s)


def test_batch_of_odd_sized_frames_equals_plain(ctx):
    """Frames whose pixel counts are not multiples of four (a partial last quad, an 8-B tail of
    accumulators) and frames of a few pixels, batched with others and with hit planes: each is
    its plain render, colour and planes alike."""
    scenes = small_scenes()[:3]
    sizes = [(3, 5), (7, 3), (65, 2), (33, 17), (2, 2), (31, 29), (96, 64)]
    sids = [ctx.upload(scenes[k % 3]) for k in range(len(sizes))]
    fids = [ctx.frame(w, h) for w, h in sizes]
    rds = [ctx.render_desc(w, h, 1, 3, flags=rt.RT_FLAG_HIT_PLANES) for w, h in sizes]
    try:
        ctx.batch(sids, fids, rds)
        got = [ctx.download(f, w, h) for f, (w, h) in zip(fids, sizes)]
        for k, (w, h) in enumerate(sizes):
            sid1, fid1 = ctx.upload(scenes[k % 3]), ctx.frame(w, h)
            try:
                ctx.render(sid1, fid1, rds[k])
                ref = ctx.download(fid1, w, h)
            finally:
                ctx.release_frame(fid1)
                ctx.release_scene(sid1)
            for key in ("rgb", "rgb8", "obj", "prim", "t"):
                np.testing.assert_array_equal(got[k][key].view(np.uint8), ref[key].view(np.uint8), err_msg=f"{key} {w}x{h}")
    finally:
        for f in fids:
            ctx.release_frame(f)
        for sd in sids:
            ctx.release_scene(sd)


@pytest.mark.parametrize("lanes", [1, 2])
def test_batch_split_over_many_waves_equals_plain(ctx, lanes):
    """Queues of 2^14 entries cut the batch into dozens of waves; with two lanes consecutive
    waves run on two workspaces and streams at once. Every frame is still its plain render."""
    scenes = [rt.SceneHost.config(3, i) for i in (0, 2, 4)] + small_scenes()[:2]
    sizes = [(160, 120), (128, 128), (96, 96), (128, 96), (100, 60)]
    sids = [ctx.upload(sc) for sc in scenes]
    fids = [ctx.frame(w, h) for w, h in sizes]
    rds = [ctx.render_desc(w, h, 1, 3) for w, h in sizes]
    try:
        t = rt.BatchTuning(128, 32, 0, 1, 8, 1, 1 << 14, 4096, 0, lanes)
        ctx.batch(sids, fids, rds, tuning=t)
        st = ctx.wait()   # the batch's counters, before plain renders replace them
        assert st.rays_primary == sum(w * h for w, h in sizes)
        for sc, fid, (w, h) in zip(scenes, fids, sizes):
            got = ctx.download(fid, w, h, planes=False)
            ref = plain_render(ctx, sc, w, h)
            np.testing.assert_array_equal(got["rgb"].view(np.uint32), ref["rgb"].view(np.uint32))
    finally:
        for f in fids:
            ctx.release_frame(f)
        for sd in sids:
            ctx.release_scene(sd)


def test_autotune_returns_offered_values_and_the_same_images(ctx):
    """The autotuner's choice is one of the values it offers, with the lane count stated, and a
    batch rendered with it gives the images of the defaults bit for bit."""
    scenes = [rt.SceneHost.config(3, i) for i in (1, 3)] + small_scenes()[:2]
    sizes = [(128, 96), (96, 96), (80, 64), (64, 64)]
    sids = [ctx.upload(sc) for sc in scenes]
    fids = [ctx.frame(w, h) for w, h in sizes]
    rds = [ctx.render_desc(w, h, 1, 3) for w, h in sizes]
    try:
        t = ctx.autotune(sids, fids, rds)
        assert (t.block, t.min_blocks) in {(128, 8), (128, 6), (64, 8), (256, 0)}, t.as_dict()
        assert t.tile in (32, 64, 128, 256) and t.dynamic in (1, 2, 3), t.as_dict()
        assert t.stack in (0, 8) and t.pixel_tile in (0, 8, 16, 32), t.as_dict()
        assert t.shadow_chunk in (0, 1024, 4096, 16384) and t.lanes in (1, 2), t.as_dict()
        assert t.wave_rays in (0, 1 << 25, 1 << 27), t.as_dict()
        images = []
        for tuning in (None, t):
            ctx.batch(sids, fids, rds, tuning=tuning)
            images.append([ctx.download(f, w, h, planes=False)["rgb"] for f, (w, h) in zip(fids, sizes)])
        for a, b in zip(*images):
            np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    finally:
        for f in fids:
            ctx.release_frame(f)
        for sd in sids:
            ctx.release_scene(sd)


def test_plain_render_after_workspace_growth():
    """A render whose frame needs a larger ray workspace than the last one re-lays the
    workspace out; the cached launch graph must follow even when the new allocation comes back
    at the old address. Each frame rendered after others must equal its render in a fresh
    context."""
    scenes = small_scenes()[:3]
    sizes = [(48, 32), (160, 120), (64, 48)]

    def render_all(c, order):
        out = {}
        for k in order:
            sid = c.upload(scenes[k])
            fid = c.frame(*sizes[k])
            c.render(sid, fid, c.render_desc(*sizes[k], 1, 3))
            out[k] = c.download(fid, *sizes[k], planes=False)["rgb"].copy()
            c.release_frame(fid)
            c.release_scene(sid)
        return out

    seq = rt.Context(0)
    try:
        got = render_all(seq, [0, 1, 2, 0])   # grows at 1; 2 and the second 0 reuse the grown layout
    finally:
        seq.close()
    for k in range(3):
        fresh = rt.Context(0)
        try:
            want = render_all(fresh, [k])[k]
        finally:
            fresh.close()
        assert np.array_equal(got[k], want), k


def test_batch_jittered_depth4_equals_plain(ctx):
    scenes = small_scenes()[:2]
    sids = [ctx.upload(s) for s in scenes]
    fids = [ctx.frame(64, 48) for _ in scenes]
    rds = [ctx.render_desc(64, 48, 4, 4, seed=7) for _ in scenes]
    try:
        ctx.batch(sids, fids, rds, tuning=rt.BatchTuning(64, 64, 0, 0, 8, 1))   # no graph, other tiles
        for sc, fid in zip(scenes, fids):
            got = ctx.download(fid, 64, 48, planes=False)
            ref = plain_render(ctx, sc, 64, 48, spp=4, level=4, seed=7)
            assert np.array_equal(got["rgb"], ref["rgb"])
    finally:
        for f in fids:
            ctx.release_frame(f)
        for s in sids:
            ctx.release_scene(s)


def mixed_requests(srv, scene_ids):
    """(scene, w, h, camera, seed) of a deterministic request mix."""
    out = []
    sizes = [(96, 64), (64, 64), (120, 90), (48, 80), (128, 72), (80, 80)]
    for k in range(12):
        sid = scene_ids[k % len(scene_ids)]
        w, h = sizes[k % len(sizes)]
        cam = rt.orbit_camera(srv.camera(sid), 30.0 * k, 10.0 + 4.0 * k, w, h)
        out.append((sid, w, h, cam, 1000 + k))
    return out


def run_alone(ctx, scenes, req, **kw):
    with rt.Server(ctx, 8 << 30, max_inflight=4, queue_rays=1 << 14, max_pixels=128 * 128, **kw) as srv:
        ids = [srv.add_scene(s) for s in scenes]
        sid, w, h, cam, seed = req
        rid = srv.submit(ids[sid], w, h, cam, seed)
        srv.drain()
        return srv.result(rid)


def test_server_request_alone_equals_in_mix(ctx):
    scenes = small_scenes()
    with rt.Server(ctx, 8 << 30, max_inflight=5, queue_rays=1 << 14, max_pixels=128 * 128) as srv:
        ids = [srv.add_scene(s) for s in scenes]
        reqs = mixed_requests(srv, ids)
        rids = []
        for k, (sid, w, h, cam, seed) in enumerate(reqs):
            rids.append(srv.submit(sid, w, h, cam, seed))
            if k % 3 == 2:
                srv.step()   # later requests arrive while earlier ones are in flight
        srv.drain()
        st = srv.stats()
        results = [srv.result(r) for r in rids]
    assert st["completed"] == len(reqs) and st["rejected"] == 0
    assert st["admitted_busy"] > 0, st            # continuous batching: admitted while others ran
    assert st["mean_wave_requests"] > 1.0, st     # waves were shared between requests
    assert st["waves"] > len(reqs), st            # 16k-entry queue: frames split over waves
    for k in (0, 4, 7, 11):
        alone = run_alone(ctx, scenes, reqs[k])
        assert np.array_equal(alone["rgb"], results[k]["rgb"]), k
        assert np.array_equal(alone["rgb8"], results[k]["rgb8"]), k
        sid, w, h, cam, seed = reqs[k]
        ref = plain_render(ctx, scenes[sid], w, h, camera=cam, seed=seed)
        assert np.array_equal(ref["rgb"], results[k]["rgb"]), k


def test_server_tuning_changes_no_image(ctx):
    """A server whose waves run another tuning (stack entries in shared memory, pixel tiles,
    shadow chunks, tiles, two lanes instead of one) gives every request the image of the default
    tuning."""
    scenes = small_scenes()[:3]
    images = []
    for tuning in (None, rt.BatchTuning(128, 64, 8, 1, 8, 1, 0, 2048, 16),
                   rt.BatchTuning(128, 32, 0, 1, 8, 1, 0, 4096, 0, 2)):
        with rt.Server(ctx, 8 << 30, max_inflight=4, queue_rays=1 << 14, max_pixels=128 * 128) as srv:
            if tuning is not None:
                srv.set_tuning(tuning)
            ids = [srv.add_scene(s) for s in scenes]
            rids = []
            for k, r in enumerate(mixed_requests(srv, ids)[:6]):
                rids.append(srv.submit(*r))
                if k % 2:
                    srv.step()   # requests finish in different waves, on both lanes
            srv.drain()
            st = srv.stats()
            images.append([srv.result(r)["rgb"] for r in rids])
        assert st["waves"] > 6, st
    for other in images[1:]:
        for a, b in zip(images[0], other):
            np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    with rt.Server(ctx, 8 << 30, max_inflight=4) as srv:
        with pytest.raises(rt.RTError) as e:
            srv.set_tuning(rt.BatchTuning(128, 32, 5, 1, 8, 1, 0, 0, 0))   # 5 stack entries: not offered
        assert e.value.code == rt.RT_ERR_INVALID
        sid = srv.add_scene(scenes[0])
        srv.submit(sid, 32, 32)
        with pytest.raises(rt.RTError) as e:   # the lane count changes only on an idle server
            srv.set_tuning(rt.BatchTuning(128, 32, 0, 1, 8, 1, 0, 0, 0, 2))
        assert e.value.code == rt.RT_ERR_BUSY
        srv.drain()
        srv.set_tuning(rt.BatchTuning(128, 32, 0, 1, 8, 1, 0, 0, 0, 2))
    # the plain mode renders with the server's tuning, leaving the context's own as it was
    before = ctx.tuning().as_dict()
    with rt.Server(ctx, 8 << 30, max_inflight=4, plain=True, max_pixels=128 * 128) as srv:
        srv.set_tuning(rt.BatchTuning(128, 32, 0, 1, 8, 1, 0, 1024, 16, 1))
        sid = srv.add_scene(scenes[0])
        sid_, w, h, cam, seed = mixed_requests(srv, [sid])[0]
        rid = srv.submit(sid, w, h, cam, seed)
        srv.drain()
        np.testing.assert_array_equal(srv.result(rid)["rgb"].view(np.uint32), images[0][0].view(np.uint32))
    assert ctx.tuning().as_dict() == before


def test_server_plain_mode_matches_batched(ctx):
    scenes = small_scenes()[:3]
    images = {}
    for plain in (False, True):
        with rt.Server(ctx, 8 << 30, max_inflight=4, plain=plain, max_pixels=128 * 128) as srv:
            ids = [srv.add_scene(s) for s in scenes]
            reqs = mixed_requests(srv, ids)[:6]
            rids = [srv.submit(*r) for r in reqs]
            srv.drain()
            images[plain] = [srv.result(r)["rgb"] for r in rids]
    for a, b in zip(images[False], images[True]):
        assert np.array_equal(a, b)


def test_server_matches_oracle(ctx):
    from oracle import port

    scene = rt.SceneHost.small(seed=31, n_spheres=6, ico_freq=4, width=64, height=48, refractive_every=3)
    with rt.Server(ctx, 4 << 30, max_inflight=2, max_pixels=64 * 64) as srv:
        sid = srv.add_scene(scene)
        rid = srv.submit(sid, 64, 48)
        srv.drain()
        got = srv.result(rid)
    ref = port.render(scene, 64, 48, spp=1, max_level=3)
    diff = np.abs(got["rgb"] - ref["rgb"]).max(axis=2)
    bad = (diff > 1e-4) & ~ref["ambiguous"]
    assert not bad.any(), int(bad.sum())


def test_server_lru_eviction_and_rebuild(ctx):
    scenes = [rt.SceneHost.config(4, i) for i in range(4)]
    sizes = []
    for s in scenes:   # device bytes of each scene (this also grows the LBVH scratch to its final size)
        sid = ctx.upload(s)
        sizes.append(ctx.device_bytes(sid))
        ctx.release_scene(sid)
    with rt.Server(ctx, 64 << 30, max_inflight=2, max_pixels=96 * 96, queue_rays=1 << 16) as big:
        ids = [big.add_scene(s) for s in scenes]
        reqs = [(ids[k % 4], 96, 64, rt.orbit_camera(big.camera(ids[k % 4]), 45.0 * k, 20.0, 96, 64), k)
                for k in range(10)]
        want = []
        for r in reqs:
            rid = big.submit(*r)
            big.drain()
            want.append(big.result(rid)["rgb"])
        assert big.stats()["evictions"] == 0
    srt = sorted(sizes)
    ctx.release_cached()   # buffers kept from earlier releases would count against the budget
    # the same wave queue size in both servers (the default one follows the budget)
    with rt.Server(ctx, 64 << 30, max_inflight=2, max_pixels=96 * 96, queue_rays=1 << 16) as probe:
        base = probe.stats()["peak_bytes"]   # slots + queues + LBVH scratch
    budget = base + srt[-1] + srt[-2] + srt[0] // 2   # the two largest fit together, all four never
    ctx.release_cached()
    with rt.Server(ctx, budget, max_inflight=2, max_pixels=96 * 96, queue_rays=1 << 16) as small:
        ids = [small.add_scene(s) for s in scenes]
        assert sum(small.resident(i) for i in ids) < 4
        got, rebuilt = [], 0
        for r in reqs:
            rid = small.submit(*r)
            small.drain()
            res = small.result(rid)
            rebuilt += res["rebuilt"]
            got.append(res["rgb"])
        st = small.stats()
    assert st["evictions"] > 0 and st["rebuilds"] > 0 and rebuilt == st["rebuilds"], st
    assert st["peak_bytes"] <= budget, (st, budget)
    for a, b in zip(want, got):
        assert np.array_equal(a, b)


def test_server_errors(ctx):
    scene = small_scenes()[0]
    with pytest.raises(rt.RTError) as e:
        rt.Server(ctx, 1 << 20)   # the wave queues alone exceed a 1 MB budget
    assert e.value.code == rt.RT_ERR_BUDGET
    with rt.Server(ctx, 4 << 30, max_inflight=2, max_pixels=64 * 64) as srv:
        sid = srv.add_scene(scene)
        with pytest.raises(rt.RTError) as e:
            srv.submit(sid + 5, 32, 32)
        assert e.value.code == rt.RT_ERR_NOT_FOUND
        with pytest.raises(rt.RTError) as e:
            srv.submit(sid, 128, 128)   # more pixels than a frame slot holds
        assert e.value.code == rt.RT_ERR_INVALID
        rid = srv.submit(sid, 32, 32)
        assert srv.result(rid) is None   # queued: not done yet
        srv.drain()
        assert srv.result(rid)["status"] == 0


def test_server_poisson_stream(ctx):
    scenes = [rt.SceneHost.config(4, i) for i in range(3)]
    out = {}
    for plain in (False, True):
        with rt.Server(ctx, 32 << 30, max_inflight=16, plain=plain, keep_images=False) as srv:
            for s in scenes:
                srv.add_scene(s)
            out[plain] = srv.run_poisson(100.0, 0.5, seed=4)
    for plain, st in out.items():
        assert st["requests"] > 10, st
        assert st["completed"] == st["requests"] and st["rejected"] == 0, st
        assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"], st
        assert st["mrays_per_s"] > 0 and st["rays"] > 0, st
    assert out[False]["requests"] == out[True]["requests"]   # same seeded stream
    assert out[False]["pixels"] == out[True]["pixels"]


def test_batch_mixes_render_modes(ctx):
    """Jobs of different test modes (and depths) share waves and equal their plain renders."""
    scene = rt.SceneHost.textured(6, 64, 64)
    modes = [rt.RT_MODE_RAYTRACE, rt.RT_MODE_NORMAL, rt.RT_MODE_SHADOW, rt.RT_MODE_REFLECT, rt.RT_MODE_DEPTH,
             rt.RT_MODE_CHECK]
    sid = ctx.upload(scene)
    fids = [ctx.frame(64, 48) for _ in modes]
    rds = [ctx.render_desc(64, 48, 2, 3, mode=m, seed=5) for m in modes]
    try:
        ctx.batch([sid] * len(modes), fids, rds)
        got = [ctx.download(f, 64, 48, planes=False)["rgb"] for f in fids]
        for m, rd, g in zip(modes, rds, got):
            ctx.render(sid, fids[0], rd)
            assert np.array_equal(ctx.download(fids[0], 64, 48, planes=False)["rgb"], g), hex(m)
    finally:
        for f in fids:
            ctx.release_frame(f)
        ctx.release_scene(sid)


def test_server_multi_sample_requests_equal_plain_renders(ctx):
    scenes = small_scenes()[:2]
    with rt.Server(ctx, 8 << 30, max_inflight=4, spp=4, max_level=4, queue_rays=1 << 15, max_pixels=96 * 96) as srv:
        ids = [srv.add_scene(s) for s in scenes]
        reqs = [(ids[k % 2], 80, 60, rt.orbit_camera(srv.camera(ids[k % 2]), 50.0 * k, 25.0, 80, 60), 900 + k)
                for k in range(4)]
        rids = [srv.submit(*r) for r in reqs]
        srv.drain()
        got = [srv.result(r)["rgb"] for r in rids]
    for (sid, w, h, cam, seed), g in zip(reqs, got):
        ref = plain_render(ctx, scenes[sid], w, h, camera=cam, spp=4, level=4, seed=seed)
        assert np.array_equal(ref["rgb"], g)



def test_cli_serves_a_short_stream():
    """The CLI's serving mode: a short Poisson stream over a few config-4 scenes completes every
    request."""
    from raytrace_gb300 import cli

    st = cli.serve(200.0, 0.25, 4, 16, False, slots=32)
    assert st["requests"] > 0 and st["completed"] == st["requests"] and st["rejected"] == 0, st
    assert st["p99_ms"] >= st["p50_ms"] > 0, st
