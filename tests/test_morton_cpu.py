"""The CPU Morton reference (oracle) against an independent numpy statement of the same code."""
import numpy as np

from oracle import port


def numpy_morton(tri):
    p = tri.reshape(-1, 3, 3).astype(np.float32)
    p0 = p[:, 0] + np.float32(0)
    a, b, c = p0, p0 + (p[:, 1] - p[:, 0]), p0 + (p[:, 2] - p[:, 0])
    mn = np.minimum(a, np.minimum(b, c))
    mx = np.maximum(a, np.maximum(b, c))
    cen = (mn + mx) * np.float32(0.5)
    smn, smx = mn.min(axis=0), mx.max(axis=0)
    emax = (smx - smn).max()   # one scale for all axes: cubic cells over the scene box
    scale = np.float32(1024) / emax if emax > 0 else np.float32(0)
    q = np.clip(((cen - smn) * scale).astype(np.int64), 0, 1023).astype(np.uint32)

    def expand(v):
        v = v & 0x3FF
        v = (v * 0x00010001) & 0xFF0000FF
        v = (v * 0x00000101) & 0x0F00F00F
        v = (v * 0x00000011) & 0xC30C30C3
        v = (v * 0x00000005) & 0x49249249
        return v.astype(np.uint32)

    code = (expand(q[:, 0]) << 2) | (expand(q[:, 1]) << 1) | expand(q[:, 2])
    perm = np.argsort(code, kind="stable").astype(np.uint32)
    return code[perm], perm


def test_morton_matches_numpy():
    rng = np.random.default_rng(0)
    tri = rng.normal(size=(5000, 9)).astype(np.float32)
    tri[100:200] = tri[100]   # duplicated triangles: equal codes keep index order
    c1, p1 = port.morton_sort(tri)
    c2, p2 = numpy_morton(tri)
    np.testing.assert_array_equal(c1, c2)
    np.testing.assert_array_equal(p1, p2)
    assert np.all(np.diff(c1.astype(np.int64)) >= 0)


def test_morton_degenerate_axis():
    tri = np.zeros((64, 9), np.float32)
    tri[:, 0::3] = np.arange(64, dtype=np.float32)[:, None]   # all on the x axis
    c1, p1 = port.morton_sort(tri)
    c2, p2 = numpy_morton(tri)
    np.testing.assert_array_equal(c1, c2)
    np.testing.assert_array_equal(p1, p2)
