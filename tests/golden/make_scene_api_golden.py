"""Generate tests/golden/scene_api/trace_ref.txt and render_ref.npz from the reference itself.

Builds oracle/_ref/rt_ref_scene_api (the reference's own Scene / Light / Camera / object
classes, compiled from its sources by oracle/ref/Makefile, driven by
tests/cpp/scene_api_sequence.inc) and stores what it prints: the return value of every call
of a fixed sequence of scene edits and the state after it, every float as its bit pattern.
Then builds oracle/_ref/rt_ref_scene_render, which builds the scene of
tests/cpp/scene_render_sequence.inc through the reference's API and renders it with the
reference's RayTracer::start in every mode (ray tracing and the eight MY_MODEL_* test modes)
for each of its scene variants, and stores those uint8 images (rows in the output's order).

    python tests/golden/make_scene_api_golden.py     # needs the reference sources (x86 host)
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(ROOT, "oracle", "_ref", "rt_ref_scene_api")
OUT = os.path.join(HERE, "scene_api", "trace_ref.txt")
RENDER_EXE = os.path.join(ROOT, "oracle", "_ref", "rt_ref_scene_render")
RENDER_OUT = os.path.join(HERE, "scene_api", "render_ref.npz")
# RayTracer::start's modes (RayTracer.h:9-18): ray tracing, then check, depth, normal, texture,
# material, shadow, reflect and refract tests
MODES = [0x80, 1, 2, 3, 4, 5, 6, 7, 8]
VARIANTS = 4   # the scenes of tests/cpp/scene_render_sequence.inc


def main() -> None:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), EXE], check=True)
    trace = subprocess.run([EXE], check=True, capture_output=True, text=True).stdout
    with open(OUT, "w") as f:
        f.write(trace)
    print(f"{OUT}: {len(trace.splitlines())} lines")

    import json
    import tempfile

    import numpy as np

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), RENDER_EXE], check=True)
    images, infos = {}, []
    with tempfile.TemporaryDirectory() as d:
        for variant in range(VARIANTS):
            for mode in MODES:
                img_p = os.path.join(d, f"ref_{variant}_{mode}.rgb8")
                info = json.loads(subprocess.run([RENDER_EXE, img_p, str(mode), str(variant)], check=True,
                                                 capture_output=True, text=True, cwd=os.path.join(HERE, "obj")).stdout)
                images[f"rgb8_v{variant}_{mode}"] = np.fromfile(img_p, np.uint8).reshape(info["height"], info["width"], 3)
                infos.append(info)
    np.savez_compressed(RENDER_OUT, meta=np.array(json.dumps(infos)), **images)
    print(f"{RENDER_OUT}: {len(images)} images ({VARIANTS} scenes x {len(MODES)} modes)")


if __name__ == "__main__":
    main()
