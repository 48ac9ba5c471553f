"""Shared test setup: the `gpu` marker, golden fixtures, a GPU context."""
from __future__ import annotations

import glob
import json
import os
import sys
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


def golden_names() -> list[str]:
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name: str):
    """(fixture dict, meta dict, SceneHost) of a golden case."""
    import raytrace_gb300 as rt

    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    meta = json.loads(str(g.pop("meta")))
    if "scene" in g:
        with tempfile.TemporaryDirectory() as d:
            p = os.path.join(d, "s.rtsc")
            g.pop("scene").tofile(p)
            scene = rt.SceneHost.load(p)
    else:
        if meta["generator"] == "obj":
            raise RuntimeError("OBJ fixtures embed their scene")
        gen = {"config": rt.SceneHost.config, "small": rt.SceneHost.small, "extras": rt.SceneHost.extras,
               "textured": rt.SceneHost.textured}[meta["generator"]]
        scene = gen(*meta["args"]).with_camera(meta["width"], meta["height"], meta["spp"], meta["max_level"], meta["seed"])
    return g, meta, scene


def scene_sha(scene) -> str:
    import hashlib

    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "s.rtsc")
        scene.save(p)
        return hashlib.sha256(open(p, "rb").read()).hexdigest()


@pytest.fixture(scope="session")
def ctx():
    import raytrace_gb300 as rt

    c = rt.Context(0)
    yield c
    c.close()
