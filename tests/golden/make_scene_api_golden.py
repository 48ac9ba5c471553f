"""Generate tests/golden/scene_api/trace_ref.txt and render_ref.npz from the reference itself.

Builds oracle/_ref/rt_ref_scene_api (the reference's own Scene / Light / Camera / object
classes, compiled from its sources by oracle/ref/Makefile, driven by
tests/cpp/scene_api_sequence.inc) and stores what it prints: the return value of every call
of a fixed sequence of scene edits and the state after it, every float as its bit pattern.
Then builds oracle/_ref/rt_ref_scene_render, which builds the scene of
tests/cpp/scene_render_sequence.inc through the reference's API and renders it with the
reference's RayTracer::start, and stores that uint8 image (rows in the output's order).

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
    with tempfile.TemporaryDirectory() as d:
        img_p = os.path.join(d, "ref.rgb8")
        info = json.loads(subprocess.run([RENDER_EXE, img_p], check=True, capture_output=True, text=True,
                                         cwd=os.path.join(HERE, "obj")).stdout)
        img = np.fromfile(img_p, np.uint8).reshape(info["height"], info["width"], 3)
    np.savez_compressed(RENDER_OUT, rgb8=img, meta=np.array(json.dumps(info)))
    print(f"{RENDER_OUT}: {info}")


if __name__ == "__main__":
    main()
