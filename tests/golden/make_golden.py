"""Generate the golden fixtures of tests/golden from the reference itself.

Runs oracle/_ref/rt_ref_harness (the reference's own RayTracer / Scene / object classes,
compiled from its sources by oracle/ref/Makefile) on seeded scenes and stores, per pixel of
the reference's 64x64-tile region: the float colour of proxyRTfrac before Color::put, the
uint8 image, and the primary hit object / primitive / distance. The CPU oracle's brute-force
check adds the mask of pixels whose reference result rests on a degenerate choice
(near-tie, octant-copy self hit, box pre-test disagreement).

Small scenes are stored with the fixture (the exact bytes of the scene file); large ones by
generator parameters plus the SHA-256 of their scene file.

    python tests/golden/make_golden.py            # needs oracle/_ref/rt_ref_harness
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import raytrace_gb300 as rt  # noqa: E402
from oracle import port  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "rt_ref_harness")

# name: (generator, args, width, height, spp, max_level, seed[, mode]); mode is RT_MODE_* /
# MY_MODEL_* (ray tracing when absent)
CASES = {
    "cfg0_128x64": ("config", (0,), 128, 64, 1, 3, 0),
    "ico8_refr_128x64": ("small", (5, 8, 8, 128, 64, 3), 128, 64, 1, 3, 5),
    "extras_128x64": ("extras", (3, 128, 64), 128, 64, 1, 3, 3),
    "refr_depth4_64x64": ("small", (7, 12, 0, 64, 64, 2), 64, 64, 1, 4, 7),
    "jitter4_64x64": ("small", (9, 10, 4, 64, 64, 2), 64, 64, 4, 4, 2),
    "cfg1_128x64": ("config", (1,), 128, 64, 1, 3, 1),
    "cfg2_64x64": ("config", (2,), 64, 64, 4, 4, 2),
    "extras_check_128x64": ("extras", (3, 128, 64), 128, 64, 1, 3, 3, 0x1),
    "extras_depth_128x64": ("extras", (3, 128, 64), 128, 64, 1, 3, 3, 0x2),
    "extras_normal_128x64": ("extras", (3, 128, 64), 128, 64, 1, 3, 3, 0x3),
    "extras_texture_128x64": ("extras", (3, 128, 64), 128, 64, 1, 3, 3, 0x4),
    "extras_material_128x64": ("extras", (3, 128, 64), 128, 64, 1, 3, 3, 0x5),
    "extras_shadow_128x64": ("extras", (3, 128, 64), 128, 64, 1, 3, 3, 0x6),
    "extras_reflect_128x64": ("extras", (3, 128, 64), 128, 64, 1, 3, 3, 0x7),
    "textured_128x64": ("textured", (6, 128, 64), 128, 64, 1, 3, 6),
    "textured_texture_128x64": ("textured", (6, 128, 64), 128, 64, 1, 3, 6, 0x4),
    "textured_material_128x64": ("textured", (6, 128, 64), 128, 64, 1, 3, 6, 0x5),
    "obj_house_128x64": ("obj", ("model.obj", "model.mtl", 128, 64), 128, 64, 1, 3, 0),
    "obj_house_texture_128x64": ("obj", ("model.obj", "model.mtl", 128, 64), 128, 64, 1, 3, 0, 0x4),
}
EMBED_LIMIT = 256 * 1024


def make_scene(gen: str, args: tuple, w: int, h: int, spp: int, lvl: int, seed: int) -> rt.SceneHost:
    if gen == "obj":   # the OBJ asset of tests/golden/obj (its texture is read relative to the cwd)
        cwd = os.getcwd()
        os.chdir(os.path.join(HERE, "obj"))
        try:
            base = rt.SceneHost.from_obj(*args)
        finally:
            os.chdir(cwd)
    else:
        base = {"config": rt.SceneHost.config, "small": rt.SceneHost.small, "extras": rt.SceneHost.extras,
                "textured": rt.SceneHost.textured}[gen](*args)
    return base.with_camera(w, h, spp, lvl, seed)


def scene_bytes(s: rt.SceneHost) -> bytes:
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "s.rtsc")
        s.save(p)
        return open(p, "rb").read()


def run_case(name: str, spec) -> None:
    gen, args, w, h, spp, lvl, seed = spec[:7]
    mode = spec[7] if len(spec) > 7 else 0x80
    scene = make_scene(gen, args, w, h, spp, lvl, seed)
    data = scene_bytes(scene)
    with tempfile.TemporaryDirectory() as d:
        sp = os.path.join(d, "scene.rtsc")
        open(sp, "wb").write(data)
        r = subprocess.run([HARNESS, sp, os.path.join(d, "out"), str(os.cpu_count() or 1), "-", str(mode)],
                           capture_output=True, text=True, check=True)
        info = json.loads(r.stdout)

        def ld(ext, dt, shp):
            return np.fromfile(os.path.join(d, "out." + ext), dt).reshape(shp)

        out = {"rgb": ld("rgb.f32", np.float32, (h, w, 3)), "rgb8": ld("rgb8", np.uint8, (h, w, 3)),
               "obj": ld("obj.i32", np.int32, (h, w)), "prim": ld("prim.i32", np.int32, (h, w)),
               "t": ld("t.f32", np.float32, (h, w))}
        if os.path.exists(os.path.join(d, "out.start.rgb8")):
            out["start_rgb8"] = ld("start.rgb8", np.uint8, (h, w, 3))
    chk = port.render(scene, w, h, spp, lvl, seed, ref_tiles=True, check=True, mode=mode)
    meta = {"generator": gen, "args": list(args), "width": w, "height": h, "spp": spp, "max_level": lvl,
            "seed": seed, "mode": mode, "scene_sha256": hashlib.sha256(data).hexdigest(), "harness": info}
    extra = {"scene": np.frombuffer(data, np.uint8)} if len(data) <= EMBED_LIMIT else {}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array(json.dumps(meta)),
                        ambiguous=chk["ambiguous"], reasons=chk["reasons"], **out, **extra)
    print(f"{name}: {w}x{h} spp={spp} lvl={lvl} ambiguous={int(chk['ambiguous'].sum())} "
          f"embedded={'scene' in extra} ref_pixel_pass={info['pixel_pass_s']:.2f}s", flush=True)


def main(names: list[str]) -> None:
    if not os.path.exists(HARNESS):
        raise SystemExit(f"{HARNESS} missing: run `make -C oracle/ref`")
    for n in names or list(CASES):
        run_case(n, CASES[n])


if __name__ == "__main__":
    main(sys.argv[1:])
