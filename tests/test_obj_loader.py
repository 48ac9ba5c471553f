"""The drop-in OBJ/MTL loader builds what the reference's own loader builds.

tests/golden/obj holds a small asset (quads with texture coordinates, triangles without,
usemtl parts, inherited material values, a map_Kd with a Windows path read as <name>.bmp, a
texture shared by two materials) and model_ref.npz, the reference's Model::loadOBJ output for
it (tests/golden/obj/make_obj_golden.py). Points, normals, texture coordinates, per-triangle
materials, material values, textures and bounds must be equal, bit for bit.
"""
import os

import numpy as np
import pytest

import raytrace_gb300 as rt

OBJ_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "obj")


def arr(ptr, n, dtype):
    return np.ctypeslib.as_array(ptr, (n,)).astype(dtype, copy=True)


@pytest.fixture
def loaded(monkeypatch):
    monkeypatch.chdir(OBJ_DIR)   # the loader reads textures relative to the working directory
    scene = rt.SceneHost.from_obj("model.obj", "model.mtl", 128, 64)
    return scene, scene.desc, np.load(os.path.join(OBJ_DIR, "model_ref.npz"))


def test_triangles_match_reference_loader(loaded):
    _, d, g = loaded
    ref = g["tris"]
    n = int(d.n_tris)
    assert n == len(ref) == 16
    p = arr(d.tri_p, 9 * n, np.float32).reshape(n, 9)
    nn = arr(d.tri_n, 9 * n, np.float32).reshape(n, 9)
    uv = arr(d.tri_uv, 6 * n, np.float32).reshape(n, 6)
    np.testing.assert_array_equal(p.view(np.uint32), ref[:, 0:9].view(np.uint32))
    np.testing.assert_array_equal(nn.view(np.uint32), ref[:, 9:18].view(np.uint32))
    np.testing.assert_array_equal(uv.view(np.uint32), ref[:, 18:24].view(np.uint32))


def test_materials_and_textures_match_reference_loader(loaded):
    _, d, g = loaded
    n = int(d.n_tris)
    obj = d.objects[0]
    assert d.n_objects == 1 and obj.type == rt.RT_OBJECT_MODEL
    base = obj.material                                   # the model's first material
    tri_mtl = arr(d.tri_mtl, n, np.int32)
    np.testing.assert_array_equal(tri_mtl - base, g["part_mtl"][g["tri_part"]])
    ref = g["mtls"]
    assert d.n_materials - base == len(ref)
    for i, r in enumerate(ref):
        m = d.materials[base + i]
        got = list(m.ambient) + list(m.diffuse) + list(m.specular) + [m.shininess, m.reflect, m.refract, m.rfr]
        want = list(r[0:3]) + list(r[4:7]) + list(r[8:11]) + list(r[12:16])
        np.testing.assert_array_equal(np.float32(got), np.float32(want), err_msg=f"material {i}")
        assert (m.texture >= 0) == (g["mtl_tex"][i] >= 0)
    # one texture, shared by two materials, with the reference's texels
    assert d.n_textures == len(g["tex_dims"]) == 1
    t = d.textures[0]
    assert [t.w, t.h] == list(g["tex_dims"][0])
    np.testing.assert_array_equal(arr(t.bgr, t.w * t.h * 3, np.uint8), g["texels"])
    shared = {d.materials[base + i].texture for i in range(len(ref)) if g["mtl_tex"][i] >= 0}
    assert shared == {0}
    np.testing.assert_array_equal(np.float32(list(obj.bmin) + list(obj.bmax)), g["bounds"])


def test_missing_file_is_an_error(monkeypatch):
    monkeypatch.chdir(OBJ_DIR)
    with pytest.raises(rt.RTError) as e:
        rt.SceneHost.from_obj("no_such.obj", "model.mtl")
    assert e.value.code == rt.RT_ERR_NOT_FOUND
