"""The drop-in Scene API behaves like the reference's, call for call and bit for bit.

tests/cpp/scene_api_sequence.inc runs one fixed sequence of scene edits (lights up to the
limit of 8 and past it, every object kind, light component and luminance changes, material
changes by preset and by colour, moves that translate objects, rotate the plane and ball-plane
frames and move lights, visibility switches, camera moves, deletes) and dumps the return value
of every call and the resulting lights, objects, materials and camera with each float as its
bit pattern. tests/golden/scene_api/trace_ref.txt is that trace from the reference's own classes
(tests/golden/make_scene_api_golden.py, Scene.cpp:83-301, 3DElement.cpp:340-635); here the
same sequence is compiled against the drop-in classes with the library's host flags and must
print the same trace. Where the reference-compiled program is present on this machine it is
run as well.

tests/cpp/scene_render_sequence.inc builds a scene through the same shared API (plane, moved
spheres with the reflective and refractive presets, a hidden sphere, a cube, a rotated ball
plane, the textured OBJ model of tests/golden/obj, moved point and parallel lights, a moved and
pitched camera), and three edge cases: an empty scene, every light off with the camera inside
a large refractive sphere, and a 200x136 frame with partial tiles.
tests/golden/scene_api/render_ref.npz holds the reference's RayTracer::start images of them
in every mode; the drop-in builds the same scene, flattens it as its RayTracer::start does
(flatten_scene), and the CPU oracle's render of that description must give the same bytes on
every pixel the oracle does not mark ambiguous.
"""
import importlib.util
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "scene_api", "trace_ref.txt")
REF_EXE = os.path.join(ROOT, "oracle", "_ref", "rt_ref_scene_api")
DROPIN_SOURCES = ["3DElement.cpp", "Basic3DObject.cpp", "Model.cpp", "Scene.cpp"]
RENDER_GOLDEN = os.path.join(ROOT, "tests", "golden", "scene_api", "render_ref.npz")
OBJ_DIR = os.path.join(ROOT, "tests", "golden", "obj")


def _host_flags() -> list[str]:
    spec = importlib.util.spec_from_file_location("rt_build", os.path.join(ROOT, "raytrace_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return [f for f in b.CXX_FLAGS if f != "-fPIC"]


@pytest.fixture(scope="module")
def dropin_trace(tmp_path_factory) -> str:
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("scene_api") / "scene_api_trace")
    srcs = [os.path.join(ROOT, "raytrace_gb300", "cpp", s) for s in DROPIN_SOURCES]
    subprocess.run(["g++", *_host_flags(), os.path.join(ROOT, "tests", "cpp", "scene_api_trace.cpp"), *srcs,
                    "-o", exe], check=True)
    return subprocess.run([exe], check=True, capture_output=True, text=True).stdout


def _first_difference(a: str, b: str) -> str:
    for i, (x, y) in enumerate(zip(a.splitlines(), b.splitlines())):
        if x != y:
            return f"line {i + 1}:\n  reference: {x}\n  drop-in:   {y}"
    return f"lengths differ: {len(a.splitlines())} vs {len(b.splitlines())} lines"


def test_dropin_scene_api_matches_reference_trace(dropin_trace):
    with open(GOLDEN) as f:
        golden = f.read()
    assert dropin_trace == golden, _first_difference(golden, dropin_trace)


def test_trace_covers_the_return_conventions(dropin_trace):
    calls = [l for l in dropin_trace.splitlines() if l.startswith("call ")]
    assert len(calls) == 49
    rets = [int(l.rsplit("->", 1)[1]) for l in calls]
    assert rets.count(255) == 2          # the ninth light, twice
    assert 0 in rets and 1 in rets       # failed and successful edits


@pytest.mark.skipif(not os.path.exists(REF_EXE), reason="reference-compiled program not built on this machine")
def test_reference_program_still_prints_the_golden_trace():
    live = subprocess.run([REF_EXE], check=True, capture_output=True, text=True).stdout
    with open(GOLDEN) as f:
        assert live == f.read()


@pytest.fixture(scope="module")
def dropin_render_scenes(tmp_path_factory):
    """variant -> SceneHost of the drop-in's flattened scene"""
    import raytrace_gb300 as rt

    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("scene_render")
    lib_dir = os.path.dirname(rt.LIB_PATH)
    exe = str(d / "scene_render_flatten")
    subprocess.run(["g++", *_host_flags(), os.path.join(ROOT, "tests", "cpp", "scene_render_flatten.cpp"), "-o", exe,
                    f"-L{lib_dir}", "-lrt_gb300", f"-Wl,-rpath,{lib_dir}", "-pthread"], check=True)
    out = {}
    for variant in range(len(VARIANTS)):
        scn = str(d / f"scene{variant}.rtsc")
        subprocess.run([exe, scn, str(variant)], check=True, capture_output=True, cwd=OBJ_DIR)   # textures: cwd
        out[variant] = rt.SceneHost.load(scn)
    return out


# the scenes of tests/cpp/scene_render_sequence.inc
VARIANTS = ["rich", "empty", "lights_off_camera_inside_sphere", "ragged_200x136"]


# ray tracing, then the check, depth, normal, texture, material, shadow, reflect and refract tests
@pytest.mark.parametrize("mode", [0x80, 1, 2, 3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("variant", range(len(VARIANTS)), ids=VARIANTS)
def test_dropin_scene_renders_like_reference(dropin_render_scenes, variant, mode):
    from oracle import port

    ref = np.load(RENDER_GOLDEN)[f"rgb8_v{variant}_{mode}"]
    h, w = ref.shape[:2]
    got = port.render(dropin_render_scenes[variant], w, h, 1, 3, 0, ref_tiles=True, check=True, mode=mode)
    th, tw = (h // 64) * 64, (w // 64) * 64   # the reference renders whole 64x64 tiles only
    amb = got["ambiguous"][:th, :tw]
    differ = np.any(got["rgb8"][:th, :tw] != ref[:th, :tw], axis=2)
    assert not (differ & ~amb).any(), f"{int((differ & ~amb).sum())} pixels differ ({int(amb.sum())} ambiguous)"
    assert amb.sum() <= 8
