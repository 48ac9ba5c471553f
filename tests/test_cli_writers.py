"""The headless image writers that replace the reference's glDrawPixels blit (main.cpp:197-208)."""
import numpy as np

from raytrace_gb300.cli import write_pfm, write_ppm


def test_ppm_is_top_down_rgb(tmp_path):
    img = np.arange(4 * 3 * 3, dtype=np.uint8).reshape(4, 3, 3)   # rows bottom-up, as rendered
    p = tmp_path / "a.ppm"
    write_ppm(str(p), img)
    data = p.read_bytes()
    head, body = data[:11], data[11:]
    assert head == b"P6\n3 4\n255\n"
    np.testing.assert_array_equal(np.frombuffer(body, np.uint8).reshape(4, 3, 3), img[::-1])


def test_pfm_keeps_floats_bottom_up(tmp_path):
    img = np.random.default_rng(1).random((2, 5, 3)).astype(np.float32)
    p = tmp_path / "a.pfm"
    write_pfm(str(p), img)
    data = p.read_bytes()
    head = b"PF\n5 2\n-1.0\n"
    assert data.startswith(head)
    np.testing.assert_array_equal(np.frombuffer(data[len(head):], "<f4").reshape(2, 5, 3), img)
