"""Host-side pieces of serving that need no GPU: the orbit camera of the request stream and
argument checks of the server entry points."""
import ctypes as C
import math

import numpy as np

import raytrace_gb300 as rt


def test_orbit_camera_reproduces_the_scene_camera():
    base = rt.SceneHost.config(4, 0).desc.camera
    el = math.degrees(math.atan2(2.0, 10.0))   # the generator's camera sits at (0, 2, -10)
    cam = rt.orbit_camera(base, 0.0, el, 320, 200)
    for f in ("position", "n", "u", "v"):
        assert np.allclose(list(getattr(cam, f)), list(getattr(base, f)), atol=2e-6), f
    assert (cam.width, cam.height) == (320, 200)
    assert cam.fovy == base.fovy and cam.znear == base.znear and cam.zfar == base.zfar


def test_orbit_camera_is_orthonormal_and_looks_at_origin():
    base = rt.SceneHost.config(4, 1).desc.camera
    r = np.linalg.norm(list(base.position))
    for az, el in [(0, 10), (90, 30), (200, 60), (359.9, 45)]:
        cam = rt.orbit_camera(base, az, el, 64, 64)
        p, n, u, v = (np.array(list(getattr(cam, f)), np.float64) for f in ("position", "n", "u", "v"))
        assert abs(np.linalg.norm(p) - r) < 1e-4
        assert np.allclose(n, -p / np.linalg.norm(p), atol=1e-6)
        for a in (n, u, v):
            assert abs(np.linalg.norm(a) - 1) < 1e-6
        assert abs(n @ u) < 1e-6 and abs(n @ v) < 1e-6 and abs(u @ v) < 1e-6
        assert abs(u[1]) < 1e-7 and v[1] > 0   # horizon level, up is up
        assert abs(math.degrees(math.asin(p[1] / r)) - el) < 1e-3


def test_server_entry_points_reject_bad_arguments():
    lib = rt.lib
    assert lib.rt_server_create(None, None, None) == rt.RT_ERR_INVALID
    assert lib.rt_server_submit(None, None, None) == rt.RT_ERR_INVALID
    assert lib.rt_server_step(None, None) == rt.RT_ERR_INVALID
    assert lib.rt_server_drain(None) == rt.RT_ERR_INVALID
    assert lib.rt_server_stats(None, None) == rt.RT_ERR_INVALID
    assert lib.rt_server_run_poisson(None, 1.0, 1.0, 0, None) == rt.RT_ERR_INVALID
    assert lib.rt_orbit_camera(None, 0.0, 0.0, 8, 8, None) == rt.RT_ERR_INVALID
    cam = rt.Camera()
    assert lib.rt_orbit_camera(C.byref(cam), 0.0, 0.0, 8, 8, C.byref(rt.Camera())) == rt.RT_ERR_INVALID  # r = 0
