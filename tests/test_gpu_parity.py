"""GPU renderer parity: against the reference's own outputs (golden fixtures) and against the
CPU oracle. Hit object / primitive ids must match exactly and colours within 1e-4 (absolute,
per FP32 channel, before Color::put) on every pixel the oracle does not mark ambiguous."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import raytrace_gb300 as rt
from conftest import ROOT, golden_names, load_golden
from oracle import port

pytestmark = pytest.mark.gpu
TOL = 1e-4


def gpu_render(ctx, scene, w, h, spp, lvl, seed, ref_tiles=True, mode=rt.RT_MODE_RAYTRACE):
    sid = ctx.upload(scene)
    fid = ctx.frame(w, h)
    flags = rt.RT_FLAG_HIT_PLANES | (rt.RT_FLAG_REF_TILES if ref_tiles else 0)
    st = ctx.render(sid, fid, ctx.render_desc(w, h, spp, lvl, mode=mode, flags=flags, seed=seed))
    out = ctx.download(fid, w, h)
    ctx.release_frame(fid)
    ctx.release_scene(sid)
    return out, st


def check_parity(out, ref, amb, h, w, max_rgb8_lsb=1):
    rh, rw = (h // 64) * 64, (w // 64) * 64
    sl = (slice(0, rh), slice(0, rw))
    a = amb[sl]
    ids_equal = (out["obj"][sl] == ref["obj"][sl]) & (out["prim"][sl] == ref["prim"][sl])
    bad_ids = ~ids_equal & ~a
    assert not bad_ids.any(), f"{int(bad_ids.sum())} unambiguous pixels hit another primitive"
    same = ids_equal & (ref["obj"][sl] >= 0)
    np.testing.assert_array_equal(out["t"][sl][same].view(np.uint32), ref["t"][sl][same].view(np.uint32))
    d = np.abs(out["rgb"][sl] - ref["rgb"][sl]).max(axis=2)
    bad = (d > TOL) & ~a
    assert not bad.any(), f"{int(bad.sum())} unambiguous pixels differ by more than {TOL} (max {d[~a].max():.3g})"
    lsb = np.abs(out["rgb8"][sl].astype(int) - ref["rgb8"][sl].astype(int)).max(axis=2)
    assert lsb[~a].max() <= max_rgb8_lsb
    return {"ambiguous": int(a.sum()), "max_rgb_diff": float(d[~a].max()) if (~a).any() else 0.0}


@pytest.mark.parametrize("name", golden_names())
def test_gpu_matches_reference_fixture(ctx, name):
    g, meta, scene = load_golden(name)
    w, h = meta["width"], meta["height"]
    out, st = gpu_render(ctx, scene, w, h, meta["spp"], meta["max_level"], meta["seed"],
                         mode=meta.get("mode", rt.RT_MODE_RAYTRACE))
    check_parity(out, g, g["ambiguous"], h, w)


@pytest.mark.parametrize("seed,n_spheres,ico,refr", [(1, 8, 0, 0), (2, 12, 6, 3), (3, 5, 10, 2), (4, 16, 3, 4)])
def test_gpu_matches_oracle_small(ctx, seed, n_spheres, ico, refr):
    w, h = 96, 80
    scene = rt.SceneHost.small(seed, n_spheres, ico, w, h, refr)
    out, _ = gpu_render(ctx, scene, w, h, 1, 3, seed, ref_tiles=False)
    ref = port.render(scene, w, h, 1, 3, seed, ref_tiles=False, check=True)
    # full frame (not only the 64x64 tiles): compare every pixel
    a = ref["ambiguous"]
    ids_equal = (out["obj"] == ref["obj"]) & (out["prim"] == ref["prim"])
    assert not (~ids_equal & ~a).any()
    d = np.abs(out["rgb"] - ref["rgb"]).max(axis=2)
    assert not ((d > TOL) & ~a).any(), d[~a].max()


@pytest.mark.parametrize("w,h", [(2, 2), (3, 5), (65, 2), (2, 70)])
def test_tiny_frames_match_oracle(ctx, w, h):
    """Frames of a few pixels, odd sizes and one-tile-wide strips: every pixel against the oracle."""
    scene = rt.SceneHost.small(5, 6, 4, w, h, 2)
    out, _ = gpu_render(ctx, scene, w, h, 1, 3, 5, ref_tiles=False)
    ref = port.render(scene, w, h, 1, 3, 5, ref_tiles=False, check=True)
    a = ref["ambiguous"]
    ids_equal = (out["obj"] == ref["obj"]) & (out["prim"] == ref["prim"])
    assert not (~ids_equal & ~a).any()
    d = np.abs(out["rgb"] - ref["rgb"]).max(axis=2)
    assert not ((d > TOL) & ~a).any(), d[~a].max()


def _without_planes(scene: rt.SceneHost, camera: rt.Camera) -> rt.SceneHost:
    """A copy of `scene` seen through `camera`, with its planes hidden: every primitive is then
    inside the LBVH, and rays that leave the scene miss everything."""
    d = rt.SceneDesc.from_buffer_copy(scene.desc)
    objs = (rt.Object * d.n_objects)()
    for k in range(d.n_objects):
        objs[k] = d.objects[k]
        if objs[k].type == rt.RT_OBJECT_PLANE:
            objs[k].show = 0
    d.objects = objs
    d.camera = camera
    out = rt.SceneHost.from_desc(d, *scene.params)
    return out


@pytest.mark.parametrize("dist,az,el", [(1.0, 0.0, 11.3), (3.5, 130.0, 35.0), (0.15, 250.0, 20.0)])
def test_cameras_outside_and_inside_the_scene_match_oracle(ctx, dist, az, el):
    """A plane-free scene (all primitives in the LBVH) from orbit cameras: the scene's own
    distance, a far camera (a small object, most rays leave the scene at once) and a camera
    inside the scene's box. Full frames against the brute-force oracle."""
    w, h = 96, 64
    base = rt.SceneHost.small(5, 10, 6, w, h, 3)
    cam = rt.orbit_camera(base.desc.camera, az, el, w, h)
    for k in range(3):
        cam.position[k] *= dist
    scene = _without_planes(base, cam)
    out, _ = gpu_render(ctx, scene, w, h, 1, 3, 0, ref_tiles=False)
    ref = port.render(scene, w, h, 1, 3, 0, ref_tiles=False, check=True)
    a = ref["ambiguous"]
    ids_equal = (out["obj"] == ref["obj"]) & (out["prim"] == ref["prim"])
    assert not (~ids_equal & ~a).any()
    d = np.abs(out["rgb"] - ref["rgb"]).max(axis=2)
    assert not ((d > TOL) & ~a).any(), d[~a].max()
    assert (ref["obj"] >= 0).any() and (ref["obj"] < 0).any()   # both hits and misses in the frame


@pytest.mark.parametrize("seed,n_spheres,ico,refr", [(6, 12, 8, 3), (7, 9, 12, 0)])
def test_clustered_hierarchy_matches_oracle(ctx, seed, n_spheres, ico, refr):
    """The clustering build gives another tree over the same leaves: the frame must still be
    the oracle's, pixel for pixel."""
    w, h = 96, 80
    scene = rt.SceneHost.small(seed, n_spheres, ico, w, h, refr)
    ctx.set_build(rt.RT_BUILD_CLUSTER)
    try:
        out, _ = gpu_render(ctx, scene, w, h, 1, 3, seed, ref_tiles=False)
    finally:
        ctx.set_build(rt.RT_BUILD_RADIX)
    ref = port.render(scene, w, h, 1, 3, seed, ref_tiles=False, check=True)
    a = ref["ambiguous"]
    ids_equal = (out["obj"] == ref["obj"]) & (out["prim"] == ref["prim"])
    assert not (~ids_equal & ~a).any()
    d = np.abs(out["rgb"] - ref["rgb"]).max(axis=2)
    assert not ((d > TOL) & ~a).any(), d[~a].max()


def test_gpu_matches_oracle_jitter_depth4(ctx):
    w, h = 64, 64
    scene = rt.SceneHost.small(21, 14, 5, w, h, 2)
    out, st = gpu_render(ctx, scene, w, h, 4, 4, 77)
    ref = port.render(scene, w, h, 4, 4, 77, ref_tiles=True, check=True)
    check_parity(out, ref, ref["ambiguous"], h, w)
    assert st.rays_primary == w * h * 4
    got = np.array([st.rays_primary, st.rays_secondary, st.rays_shadow])
    if ref["ambiguous"].any():   # a near-tie may change the ray tree below that pixel
        assert np.all(np.abs(got - ref["counts"]) <= 1e-3 * ref["counts"] + 64)
    else:
        np.testing.assert_array_equal(ref["counts"], got)


def test_ray_counts_match_oracle(ctx):
    w, h = 128, 128
    scene = rt.SceneHost.config(0).with_camera(w, h)
    _, st = gpu_render(ctx, scene, w, h, 1, 3, 0, ref_tiles=False)
    ref = port.render(scene, w, h, 1, 3, 0, check=False)
    assert [st.rays_primary, st.rays_secondary, st.rays_shadow] == ref["counts"].tolist()


def test_config1_full_frame(ctx):
    """81,920-triangle mesh at 1024x768: every mismatch must be a pixel the oracle marks."""
    scene = rt.SceneHost.config(1)
    w, h = 1024, 768
    out, _ = gpu_render(ctx, scene, w, h, 1, 3, 1)
    ref = port.render(scene, w, h, 1, 3, 1, ref_tiles=True, check=False)
    d = np.abs(out["rgb"] - ref["rgb"]).max(axis=2)
    bad = (d > TOL) | (out["obj"] != ref["obj"]) | (out["prim"] != ref["prim"])
    assert bad.mean() < 1e-3, bad.sum()
    ys, xs = np.nonzero(bad)
    tiles = sorted({(y // 64) * (w // 64) + x // 64 for y, x in zip(ys, xs)})
    if tiles:
        chk = port.render(scene, w, h, 1, 3, 1, ref_tiles=True, check=True, tiles=tiles)
        unexplained = bad & ~chk["ambiguous"]
        assert not unexplained.any(), list(zip(*np.nonzero(unexplained)))[:10]


def test_deterministic_and_order_independent(ctx):
    scene = rt.SceneHost.config(1).with_camera(256, 192)
    a, _ = gpu_render(ctx, scene, 256, 192, 1, 3, 1)
    b, _ = gpu_render(ctx, scene, 256, 192, 1, 3, 1)
    np.testing.assert_array_equal(a["rgb"].view(np.uint32), b["rgb"].view(np.uint32))


# (stack entries in shared memory, shadow chunk, register cap, pixel tile, work mode: 1 tiles from
# one counter, 2 static stride, 3 per-SM shares first)
TUNINGS = [(0, 0, 8, 0, 1), (8, 0, 8, 0, 1), (8, 64, 8, 16, 3), (8, 2048, 8, 8, 2), (0, 64, 6, 7, 3),
           (0, 32768, 0, 32, 1), (0, 4096, 8, 64, 3), (0, 0, 0, 0, 3)]


@pytest.mark.parametrize("stack,chunk,cap,ptile,work", TUNINGS)
def test_tuning_variants_give_the_same_image(ctx, stack, chunk, cap, ptile, work):
    """Traversal stack entries in shared memory (0, 8), shadow work in light-major chunks,
    register caps, the pixel tiles primary rays are traced in (frames whose sides are not
    multiples of the tile included) and how warps share the rays (one counter, static stride,
    per-SM shares then a common pool then stealing) change only how the work runs: every
    variant's frame is the default's bit for bit, through the plain path and through the batch
    path, on a deep jittered frame with refraction (long traversal stacks) and on a config-3
    mesh."""
    scene = rt.SceneHost.small(21, 14, 12, 96, 64, 2)
    mesh = rt.SceneHost.config(3, 4)
    want = [gpu_render(ctx, scene, 96, 64, 4, 4, 77, ref_tiles=False)[0],
            gpu_render(ctx, mesh, 128, 96, 1, 3, 0, ref_tiles=False)[0]]
    ctx.set_tuning(rt.BatchTuning(128 if cap else 256, 32, stack, 1, cap, work, 0, chunk, ptile))
    try:
        got = [gpu_render(ctx, scene, 96, 64, 4, 4, 77, ref_tiles=False)[0],
               gpu_render(ctx, mesh, 128, 96, 1, 3, 0, ref_tiles=False)[0]]
    finally:
        ctx.set_tuning(None)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g["rgb"].view(np.uint32), w["rgb"].view(np.uint32))
        np.testing.assert_array_equal(g["obj"], w["obj"])
    sids = [ctx.upload(scene), ctx.upload(mesh)]
    fids = [ctx.frame(96, 64), ctx.frame(128, 96)]
    rds = [ctx.render_desc(96, 64, 4, 4, flags=rt.RT_FLAG_HIT_PLANES, seed=77),
           ctx.render_desc(128, 96, 1, 3, flags=rt.RT_FLAG_HIT_PLANES)]
    try:
        ctx.batch(sids, fids, rds, tuning=rt.BatchTuning(128 if cap else 256, 64, stack, 1, cap, work, 0, chunk, ptile))
        for f, (w, h), ref in zip(fids, [(96, 64), (128, 96)], want):
            got_b = ctx.download(f, w, h)
            np.testing.assert_array_equal(got_b["rgb"].view(np.uint32), ref["rgb"].view(np.uint32))
            np.testing.assert_array_equal(got_b["obj"], ref["obj"])
    finally:
        for f in fids:
            ctx.release_frame(f)
        for s in sids:
            ctx.release_scene(s)


def test_profile_reports_kernel_times_and_idle_shares(ctx):
    """RT_FLAG_PROFILE: event times per kernel kind and, from each warp's start and end stamps,
    the share of the traversal and shading launches' warp time spent idle (before a block
    started or after a warp ran out of work); the image is the unprofiled one."""
    scene = rt.SceneHost.config(1).with_camera(256, 192)
    plain, _ = gpu_render(ctx, scene, 256, 192, 1, 3, 1)
    sid = ctx.upload(scene)
    fid = ctx.frame(256, 192)
    try:
        st = ctx.render(sid, fid, ctx.render_desc(256, 192, 1, 3, flags=rt.RT_FLAG_PROFILE | rt.RT_FLAG_HIT_PLANES))
        prof = ctx.download(fid, 256, 192)
        d = st.as_dict()
        for k in ("extend", "shade", "shadow"):
            assert d["kernel_ms"][k] > 0 and d["kernel_launches"][k] == 4
            assert 0.0 < d["kernel_idle"][k] < 1.0, d["kernel_idle"]
        st2 = ctx.render(sid, fid, ctx.render_desc(256, 192, 1, 3))   # unprofiled: no idle shares
        assert all(v == 0.0 for v in st2.as_dict()["kernel_idle"].values())
    finally:
        ctx.release_frame(fid)
        ctx.release_scene(sid)
    np.testing.assert_array_equal(prof["rgb"].view(np.uint32), plain["rgb"].view(np.uint32))


def test_render_host_equals_device_path(ctx):
    scene = rt.SceneHost.small(31, 10, 6, 128, 96, 3)
    out, _ = gpu_render(ctx, scene, 128, 96, 1, 3, 0, ref_tiles=False)
    rgb, rgb8, st = ctx.render_host(scene, ctx.render_desc(128, 96, 1, 3), 128, 96)
    np.testing.assert_array_equal(rgb.view(np.uint32), out["rgb"].view(np.uint32))
    np.testing.assert_array_equal(rgb8, out["rgb8"])


def test_invalid_requests_fail_cleanly(ctx):
    scene = rt.SceneHost.small(3, 4, 0, 64, 64)
    sid = ctx.upload(scene)
    fid = ctx.frame(32, 32)
    with pytest.raises(rt.RTError) as e:
        ctx.render(sid, fid, ctx.render_desc(64, 64, 1, 3))   # frame size mismatch
    assert e.value.code == rt.RT_ERR_INVALID
    with pytest.raises(rt.RTError):
        ctx.render(sid, fid, ctx.render_desc(32, 32, 1, 9))   # depth outside 0..4
    with pytest.raises(rt.RTError) as e:
        ctx.render(sid + 1000, fid, ctx.render_desc(32, 32, 1, 3))
    assert e.value.code == rt.RT_ERR_NOT_FOUND
    ctx.release_frame(fid)
    ctx.release_scene(sid)


def test_dropin_cpp_api(ctx):
    """Scene / RayTracer C++ API: RayTracer::start output equals the C ABI render of the
    flattened scene, and matches the oracle within one uint8 step off ambiguous pixels."""
    lib_dir = os.path.dirname(rt.LIB_PATH)
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "dropin_test")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(ROOT, "tests", "cpp", "dropin_test.cpp"),
                        "-o", exe, f"-L{lib_dir}", "-lrt_gb300", f"-Wl,-rpath,{lib_dir}", "-pthread"], check=True)
        img_p, scn_p = os.path.join(d, "out.rgb8"), os.path.join(d, "s.rtsc")
        subprocess.run([exe, img_p, scn_p], check=True, capture_output=True)
        w, h = 192, 128
        img = np.fromfile(img_p, np.uint8).reshape(h, w, 3)
        scene = rt.SceneHost.load(scn_p)
    out, _ = gpu_render(ctx, scene, w, h, 1, 3, 0)
    np.testing.assert_array_equal(img[:128, :192], out["rgb8"][:128, :192])
    ref = port.render(scene, w, h, 1, 3, 0, ref_tiles=True, check=True)
    check_parity(out, ref, ref["ambiguous"], h, w)
    assert scene.desc.objects[4].show == 0


def test_morton_sort_bit_exact(ctx):
    scene = rt.SceneHost.config(1)
    tri = scene.tri_points()
    for data in (tri, np.repeat(tri[:1000], 3, axis=0), np.random.default_rng(5).normal(size=(200000, 9)).astype(np.float32)):
        c_gpu, p_gpu = ctx.morton_sort(data)
        c_cpu, p_cpu = port.morton_sort(data)
        np.testing.assert_array_equal(c_gpu, c_cpu)
        np.testing.assert_array_equal(p_gpu, p_cpu)


@pytest.mark.parametrize("build", [rt.RT_BUILD_RADIX, rt.RT_BUILD_CLUSTER])
def test_lbvh_invariants(ctx, build):
    """Both hierarchies: leaves (triangles and spheres) all reachable exactly once, child boxes
    inside parent boxes, depth <= 63 (the traversal stack's bound), and every leaf box contains
    its primitive."""
    scene = rt.SceneHost.config(3, 5)
    ctx.set_build(build)
    try:
        sid = ctx.upload(scene)
    finally:
        ctx.set_build(rt.RT_BUILD_RADIX)
    nodes, perm = ctx.bvh(sid)
    ctx.release_scene(sid)
    d = scene.desc
    n_tri = d.n_tris
    spheres = [d.objects[k] for k in range(d.n_objects) if d.objects[k].type == rt.RT_OBJECT_SPHERE]
    L = n_tri + len(spheres)
    assert nodes.shape[0] == 2 * L - 1
    is_sph = (perm & 0x80000000) != 0
    assert sorted(perm[~is_sph].tolist()) == list(range(n_tri))   # single model: ids 0..n-1
    assert sorted((perm[is_sph] & 0x7FFFFFFF).tolist()) == list(range(len(spheres)))
    lo, hi = nodes[:, :3], nodes[:, 4:7]
    left = nodes[:, 3].view(np.int32)
    right = nodes[:, 7].view(np.int32)
    seen = np.zeros(2 * L - 1, np.int32)
    stack = [0]
    depth = {0: 0}
    while stack:
        k = stack.pop()
        seen[k] += 1
        if k >= L - 1:
            continue
        for c in (left[k], right[k]):
            assert 0 <= c < 2 * L - 1
            assert np.all(lo[c] >= lo[k]) and np.all(hi[c] <= hi[k])
            depth[c] = depth[k] + 1
            stack.append(c)
    assert np.all(seen == 1), "every node reachable exactly once"
    assert max(depth.values()) <= 63
    tri = scene.tri_points().reshape(-1, 3, 3)
    leaf_lo, leaf_hi = lo[L - 1:], hi[L - 1:]
    t_idx = np.nonzero(~is_sph)[0]
    pts = tri[perm[t_idx]]
    assert np.all(pts.min(axis=1) >= leaf_lo[t_idx]) and np.all(pts.max(axis=1) <= leaf_hi[t_idx])
    for k in np.nonzero(is_sph)[0]:
        sph = spheres[perm[k] & 0x7FFFFFFF]
        c, r = np.array(list(sph.position), np.float32), np.float32(sph.radius)
        assert np.all(c - r >= leaf_lo[k]) and np.all(c + r <= leaf_hi[k])


def _tree_depth(nodes: np.ndarray, L: int) -> int:
    left, right = nodes[:, 3].view(np.int32), nodes[:, 7].view(np.int32)
    seen = np.zeros(2 * L - 1, np.int32)
    stack, deepest = [(0, 0)], 0
    while stack:
        k, dpt = stack.pop()
        seen[k] += 1
        deepest = max(deepest, dpt)
        if k < L - 1:
            stack += [(int(left[k]), dpt + 1), (int(right[k]), dpt + 1)]
    assert np.all(seen == 1)
    return deepest


def test_clustering_deeper_than_the_stack_falls_back_to_the_radix_tree(ctx):
    """Triangles at x = 2^k: each clustering round merges only the lowest pair, which would
    make a chain as deep as the triangle count, beyond the traversal stack's bound of 63 levels.
    The build must hand back the radix tree instead, a valid tree of bounded depth."""
    scene = rt.SceneHost.small(seed=41, n_spheres=0, ico_freq=2, width=32, height=32, refractive_every=0)
    d = scene.desc
    n = d.n_tris
    assert 64 < n < 120
    p = np.ctypeslib.as_array(d.tri_p, shape=(n * 9,)).reshape(n, 3, 3)
    for k in range(n):
        s = np.float32(2.0) ** k
        p[k] = [[s, 0, 0], [s * np.float32(1.001), 0, 0], [s, 0, s * np.float32(0.001)]]
    ctx.set_build(rt.RT_BUILD_CLUSTER)
    try:
        sid = ctx.upload(scene)
    finally:
        ctx.set_build(rt.RT_BUILD_RADIX)
    nodes, _ = ctx.bvh(sid)
    ctx.release_scene(sid)
    assert _tree_depth(nodes, n) <= 63


def test_cancel_stops_a_render_and_the_next_render_is_whole(ctx):
    """rt_cancel lands on the device flag while the render runs; the render reports
    RT_ERR_CANCELLED and the next render is complete and unaffected."""
    w, h = 1920, 1080
    scene = rt.SceneHost.config(2)
    sid = ctx.upload(scene)
    fid = ctx.frame(w, h)
    try:
        small = ctx.render_desc(w, h, 1, 2, seed=3)
        ctx.render(sid, fid, small)
        want = ctx.download(fid, w, h, planes=False)["rgb"]
        ctx.render(sid, fid, ctx.render_desc(w, h, 16, 4, seed=2), wait=False)   # ~40 ms of work
        assert rt.lib.rt_cancel(ctx.handle) == 0
        with pytest.raises(rt.RTError) as e:
            ctx.wait()
        assert e.value.code == rt.RT_ERR_CANCELLED
        ctx.render(sid, fid, small)
        np.testing.assert_array_equal(ctx.download(fid, w, h, planes=False)["rgb"], want)
    finally:
        ctx.release_frame(fid)
        ctx.release_scene(sid)


def test_cancel_mark_orders_cancels_against_renders(ctx):
    """A cancel made after the mark ends rt_render_host_since even though it came before the
    call; a cancel made before a render began (rt_render, rt_render_host) does not end it."""
    import ctypes

    scene = rt.SceneHost.small(seed=9, n_spheres=6, ico_freq=8, width=96, height=64, refractive_every=3)
    rd = ctx.render_desc(96, 64, 1, 3)
    rgb8 = np.zeros((64, 96, 3), np.uint8)
    st = rt.RenderStats()
    mark = rt.lib.rt_cancel_mark(ctx.handle)
    assert rt.lib.rt_cancel(ctx.handle) == 0
    assert rt.lib.rt_cancel_mark(ctx.handle) == mark + 1
    rc = rt.lib.rt_render_host_since(ctx.handle, mark, scene.desc_ptr(), ctypes.byref(rd),
                                     rgb8.ctypes.data_as(ctypes.c_void_p), None, ctypes.byref(st))
    assert rc == rt.RT_ERR_CANCELLED
    assert not rgb8.any()
    # the same cancel is older than these calls: both complete
    _, got8, _ = ctx.render_host(scene, rd, 96, 64)
    out, _ = gpu_render(ctx, scene, 96, 64, 1, 3, 0, ref_tiles=False)
    np.testing.assert_array_equal(got8, out["rgb8"])
    rc = rt.lib.rt_render_host_since(ctx.handle, rt.lib.rt_cancel_mark(ctx.handle), scene.desc_ptr(), ctypes.byref(rd),
                                     rgb8.ctypes.data_as(ctypes.c_void_p), None, ctypes.byref(st))
    assert rc == rt.RT_OK
    np.testing.assert_array_equal(rgb8, out["rgb8"])


def test_dropin_stop_right_after_start_cancels_that_render():
    """RayTracer::stop() at once after start(): the render ends (RT_ERR_CANCELLED) sooner than a
    whole render takes and leaves `output` as start() set it; a stop() made with nothing running
    does not affect the next start()."""
    import json

    lib_dir = os.path.dirname(rt.LIB_PATH)
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "dropin_stop_test")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                        os.path.join(ROOT, "tests", "cpp", "dropin_stop_test.cpp"), "-o", exe, f"-L{lib_dir}",
                        "-lrt_gb300", f"-Wl,-rpath,{lib_dir}", "-pthread"], check=True)
        r = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=300)
    res = json.loads(r.stdout.strip().splitlines()[-1])
    print("dropin stop", res)
    assert res["full_status"] == rt.RT_OK
    assert res["stop_status"] == rt.RT_ERR_CANCELLED
    assert res["untouched"] == 1
    assert res["stop_s"] < res["full_s"]
    assert res["after_status"] == rt.RT_OK and res["written"] == 1


@pytest.mark.parametrize("mode", [rt.RT_MODE_DEPTH, rt.RT_MODE_NORMAL, rt.RT_MODE_TEXTURE, rt.RT_MODE_MATERIAL,
                                  rt.RT_MODE_SHADOW, rt.RT_MODE_REFLECT, rt.RT_MODE_CHECK])
def test_render_modes_full_frame_match_oracle(ctx, mode):
    """Every test mode of the reference on the full frame (not only its 64x64 tiles)."""
    w, h = 100, 70
    scene = rt.SceneHost.textured(6, w, h)
    out, _ = gpu_render(ctx, scene, w, h, 1, 3, 6, ref_tiles=False, mode=mode)
    ref = port.render(scene, w, h, 1, 3, 6, ref_tiles=False, check=True, mode=mode)
    a = ref["ambiguous"]
    d = np.abs(out["rgb"] - ref["rgb"]).max(axis=2)
    assert not ((d > TOL) & ~a).any(), (mode, float(d[~a].max()))


def test_out_of_range_triangle_material_is_rejected(ctx):
    """The LBVH build checks every triangle's material index on the device; the upload fails."""
    scene = rt.SceneHost.small(seed=40, n_spheres=2, ico_freq=3, width=32, height=32, refractive_every=0)
    d = scene.desc
    assert d.n_tris > 0
    d.tri_mtl[5] = d.n_materials + 7
    with pytest.raises(rt.RTError) as e:
        ctx.upload(scene)
    assert e.value.code == rt.RT_ERR_INVALID
    d.tri_mtl[5] = 0
    sid = ctx.upload(scene)   # a valid scene still uploads
    ctx.release_scene(sid)



# the scenes of tests/cpp/scene_render_sequence.inc: built through the Scene API the drop-in
# shares with the reference, flattened as the drop-in's RayTracer::start does
API_SCENES = ["rich", "empty", "lights_off_camera_inside_sphere", "ragged_200x136"]


@pytest.fixture(scope="module")
def api_scenes(tmp_path_factory):
    lib_dir = os.path.dirname(rt.LIB_PATH)
    d = tmp_path_factory.mktemp("api_scenes")
    exe = str(d / "scene_render_flatten")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    os.path.join(ROOT, "tests", "cpp", "scene_render_flatten.cpp"), "-o", exe, f"-L{lib_dir}",
                    "-lrt_gb300", f"-Wl,-rpath,{lib_dir}", "-pthread"], check=True)
    out = []
    for v in range(len(API_SCENES)):
        p = str(d / f"s{v}.rtsc")
        subprocess.run([exe, p, str(v)], check=True, capture_output=True, cwd=os.path.join(ROOT, "tests", "golden", "obj"))
        out.append(rt.SceneHost.load(p))
    return out


@pytest.mark.parametrize("mode", [rt.RT_MODE_RAYTRACE, 1, 2, 3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("variant", range(len(API_SCENES)), ids=API_SCENES)
def test_api_built_scenes_match_oracle_and_reference(ctx, api_scenes, variant, mode):
    """Scenes built through the shared Scene API (including an empty scene, every light off with
    the camera inside a sphere, and partial tiles), in every RayTracer::start mode: the GPU
    matches the CPU oracle (ids, distances, colour within the tolerance) and the reference's
    own start() image (tests/golden/scene_api/render_ref.npz) within one uint8 step."""
    scene = api_scenes[variant]
    ref_img = np.load(os.path.join(ROOT, "tests", "golden", "scene_api", "render_ref.npz"))[f"rgb8_v{variant}_{mode}"]
    h, w = ref_img.shape[:2]
    out, _ = gpu_render(ctx, scene, w, h, 1, 3, 0, mode=mode)
    ref = port.render(scene, w, h, 1, 3, 0, ref_tiles=True, check=True, mode=mode)
    check_parity(out, ref, ref["ambiguous"], h, w)
    th, tw = (h // 64) * 64, (w // 64) * 64
    lsb = np.abs(out["rgb8"][:th, :tw].astype(int) - ref_img[:th, :tw].astype(int)).max(axis=2)
    assert lsb[~ref["ambiguous"][:th, :tw]].max() <= 1
