"""The renderer's device-side limits fire and are reported, with no fault and no hang.

* A hierarchy whose root references itself (a cycle among valid node indices, so nothing is
  read outside the tree): every traversal reaching it stops at the visit limit or the stack
  bound, the render returns RT_ERR_CUDA with the "corrupt LBVH" message, and the context keeps
  working.
* Ray queues far smaller than the frame: the first attempt overflows, the render is retried
  with larger queues, and the frame equals the one rendered with queues of the default size.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import raytrace_gb300 as rt

pytestmark = pytest.mark.gpu


def _render(ctx, scene, w, h, level=3):
    sid = ctx.upload(scene)
    fid = ctx.frame(w, h)
    try:
        st = ctx.render(sid, fid, ctx.render_desc(w, h, 1, level))
        return ctx.download(fid, w, h, planes=False), st
    finally:
        ctx.release_frame(fid)
        ctx.release_scene(sid)


def test_cyclic_hierarchy_stops_at_the_visit_limit_and_is_reported(ctx):
    scene = rt.SceneHost.small(seed=3, n_spheres=4, ico_freq=6, width=8, height=8, refractive_every=0)
    sid = ctx.upload(scene)
    fid = ctx.frame(8, 8)
    try:
        bad = (C.c_int32 * 4)(0, 0, 0, 0)   # the root's four slots lead back to the root
        assert rt.lib.rt_scene_test_set_node_refs(ctx.handle, sid, 0, bad) == rt.RT_OK
        out_of_tree = (C.c_int32 * 4)(0, 0, 0, 1 << 30)
        assert rt.lib.rt_scene_test_set_node_refs(ctx.handle, sid, 0, out_of_tree) == rt.RT_ERR_INVALID
        with pytest.raises(rt.RTError) as e:
            ctx.render(sid, fid, ctx.render_desc(8, 8, 1, 0))
        assert e.value.code == rt.RT_ERR_CUDA
        msg = rt.lib.rt_last_error(ctx.handle).decode()
        assert "corrupt LBVH" in msg, msg
        flags = int(msg.rsplit("0x", 1)[1].rstrip(")"), 16)
        assert flags & 2, msg   # the visit limit ended the loop
    finally:
        ctx.release_frame(fid)
        ctx.release_scene(sid)
    # the context is usable: a valid scene renders as in a fresh context
    good = rt.SceneHost.small(seed=4, n_spheres=5, ico_freq=4, width=32, height=32, refractive_every=2)
    got, _ = _render(ctx, good, 32, 32)
    with rt.Context(0) as fresh:
        want, _ = _render(fresh, good, 32, 32)
    np.testing.assert_array_equal(got["rgb"].view(np.uint32), want["rgb"].view(np.uint32))


def test_overflowing_queue_is_retried_and_the_frame_is_whole():
    scene = rt.SceneHost.small(seed=8, n_spheres=12, ico_freq=6, width=64, height=64, refractive_every=2)
    with rt.Context(0) as small:   # a fresh context: its workspace starts at the hook's size
        assert rt.lib.rt_ctx_test_queue_entries(small.handle, 1024) == rt.RT_OK
        got, st = _render(small, scene, 64, 64)
    assert st.overflow_retries >= 1
    with rt.Context(0) as fresh:
        want, st2 = _render(fresh, scene, 64, 64)
    assert st2.overflow_retries == 0
    np.testing.assert_array_equal(got["rgb"].view(np.uint32), want["rgb"].view(np.uint32))
    np.testing.assert_array_equal(got["rgb8"], want["rgb8"])
    assert (st.rays_primary, st.rays_secondary, st.rays_shadow) == (st2.rays_primary, st2.rays_secondary,
                                                                     st2.rays_shadow)
