"""Seeded scene generators: sizes, determinism and the scene file round trip."""
import os
import tempfile

import numpy as np
import pytest

import raytrace_gb300 as rt
from conftest import scene_sha


def test_config_sizes():
    s0 = rt.SceneHost.config(0)
    assert s0.desc.n_objects == 9 and s0.desc.n_lights == 2 and s0.desc.n_tris == 0
    assert (s0.desc.camera.width, s0.desc.camera.height) == (512, 512)
    s1 = rt.SceneHost.config(1)
    assert s1.desc.n_tris == 81920 and (s1.desc.camera.width, s1.desc.camera.height) == (1024, 768)
    assert s1.params == (1, 3, 1)


def test_config2_terrain():
    s2 = rt.SceneHost.config(2)
    d = s2.desc
    assert d.n_tris == 2 * 1023 * 1023
    assert d.n_objects == 65 and d.n_lights == 4
    refr = [d.materials[d.objects[k].material].refract for k in range(1, 65)]
    assert sum(1 for r in refr if r > 0.01) == 16   # 25% refractive
    assert s2.params == (4, 4, 2)


def test_config3_population():
    tris = []
    for k in range(12):
        d = rt.SceneHost.config(3, k).desc
        tris.append(d.n_tris)
        assert d.n_objects == 17
        assert (d.camera.width, d.camera.height) in [(256, 256), (512, 512), (1024, 768), (1920, 1080)]
    assert min(tris) >= 980 and max(tris) <= 500000


def test_determinism():
    for cfg, idx in [(0, 0), (1, 0), (3, 7), (4, 3)]:
        assert scene_sha(rt.SceneHost.config(cfg, idx)) == scene_sha(rt.SceneHost.config(cfg, idx))


def test_save_load_roundtrip():
    s = rt.SceneHost.extras(4, 96, 64)
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "x.rtsc")
        s.save(p)
        t = rt.SceneHost.load(p)
        assert scene_sha(t) == scene_sha(s)
        assert t.params == s.params


def test_camera_basis_orthonormal():
    c = rt.SceneHost.config(0).desc.camera
    u, v, n = (np.array(list(x), np.float64) for x in (c.u, c.v, c.n))
    for a in (u, v, n):
        assert abs(np.linalg.norm(a) - 1) < 1e-6
    assert abs(u @ v) < 1e-6 and abs(u @ n) < 1e-6 and abs(v @ n) < 1e-6


def test_mesh_parts_respect_int16_limit():
    # the reference numbers a part's triangles with int16_t; 81920 triangles need 3 parts
    d = rt.SceneHost.config(1).desc
    ids = np.ctypeslib.as_array(d.tri_id, shape=(d.n_tris,))
    assert ids[-1] == 81919 and ids.min() == 0
