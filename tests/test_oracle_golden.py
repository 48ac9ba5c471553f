"""The CPU oracle against the reference's own outputs (golden fixtures from oracle/_ref)."""
import platform

import numpy as np
import pytest

from conftest import golden_names, load_golden, scene_sha
from oracle import port

X86 = platform.machine() in ("x86_64", "AMD64")


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference(name):
    g, meta, scene = load_golden(name)
    assert scene_sha(scene) == meta["scene_sha256"], "scene generator output changed"
    w, h = meta["width"], meta["height"]
    r = port.render(scene, w, h, meta["spp"], meta["max_level"], meta["seed"], ref_tiles=True, check=False,
                    mode=meta.get("mode", 0x80))
    rh, rw = (h // 64) * 64, (w // 64) * 64
    sl = (slice(0, rh), slice(0, rw))
    np.testing.assert_array_equal(r["obj"][sl], g["obj"][sl])
    np.testing.assert_array_equal(r["prim"][sl], g["prim"][sl])
    np.testing.assert_array_equal(r["t"][sl].view(np.uint32), g["t"][sl].view(np.uint32))
    if X86:   # same libm as the fixture run: bit-exact colour
        np.testing.assert_array_equal(r["rgb"][sl].view(np.uint32), g["rgb"][sl].view(np.uint32))
        np.testing.assert_array_equal(r["rgb8"][sl], g["rgb8"][sl])
    else:
        np.testing.assert_allclose(r["rgb"][sl], g["rgb"][sl], atol=1e-6)


@pytest.mark.parametrize("name", [n for n in golden_names()])
def test_reference_start_equals_pixel_pass(name):
    """RayTracer::start's own uint8 output equals Color::put of the per-pixel colours."""
    g, meta, _ = load_golden(name)
    if "start_rgb8" not in g:
        pytest.skip("multi-sample case: start() renders one sample")
    np.testing.assert_array_equal(g["start_rgb8"], g["rgb8"])


def test_fixture_ambiguity_is_rare():
    for name in golden_names():
        g, meta, _ = load_golden(name)
        frac = g["ambiguous"].mean()
        assert frac < 0.01, f"{name}: {frac:.3%} ambiguous pixels"


def test_oracle_fp64_close_to_fp32():
    """FP32 render error against the FP64 re-render of the same algorithm, on config 0."""
    g, meta, scene = load_golden("cfg0_128x64")
    w, h = meta["width"], meta["height"]
    r32 = port.render(scene, w, h, 1, 3, 0, ref_tiles=True, check=True)
    r64 = port.render(scene, w, h, 1, 3, 0, ref_tiles=True, fp64=True)
    same = (r32["obj"] == r64["obj"]) & ~r32["ambiguous"]
    err = np.abs(r32["rgb"].astype(np.float64) - r64["rgb"]).max(axis=2)[same]
    assert np.percentile(err, 99) < 1e-4
