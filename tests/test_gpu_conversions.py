"""The kernels' integer-exact replacements of FP64 expressions give the FP64 bits.

Ray generation computes (float)((double)X * dp), frame resolve (float)((double)acc * 2^-32/spp)
and colour accumulation llrint(v * 2^32) without FP64 instructions (slow on GB300). numpy's
float64 arithmetic is the reference: every result must be bit-identical.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dp_of(fovy_deg: float, height: int) -> float:
    return math.tan(fovy_deg * 3.1415926535897932384 / 360) / (height // 2)


def multipliers():
    ds = [dp_of(f, h) for f in (30.0, 45.0, 60.0, 90.0, 120.0) for h in (48, 64, 768, 1080, 2048)]
    ds += [dp_of(60.0, 1080) * 2.0 ** -24]                          # jittered ray generation
    ds += [1.0 / 4294967296.0 / spp for spp in (1, 2, 3, 4, 5, 7, 16, 1000)]   # resolve scale
    ds += [1.0, 0.1, 3.0e-7, 123456.789]
    return ds


def inputs(rng, n):
    x = np.concatenate([
        np.arange(-1100, 1100, dtype=np.int64),                                   # pixel offsets
        rng.integers(-8192, 8192, n) * 16777216 + rng.integers(0, 1 << 24, n),    # jittered offsets
        rng.integers(0, 1 << 40, n),                                              # colour sums
        -rng.integers(0, 1 << 45, n),
        rng.integers((1 << 53) - 4096, (1 << 53) + 4096, n),                      # around 2^53
        rng.integers(1 << 60, 1 << 62, n),
        np.array([0, 1, -1, (1 << 63) - 1, -(1 << 63) + 1], np.int64),
    ])
    v = np.concatenate([
        rng.standard_normal(x.size // 2).astype(np.float32),
        (rng.random(x.size - x.size // 2) * 2.0 ** rng.integers(-40, 30, x.size - x.size // 2)).astype(np.float32),
    ])
    v[:8] = [0.0, -0.0, 2.0 ** -33, 2.0 ** -32 * 1.5, 2.0 ** -32 * 2.5, -2.0 ** -33, 1e-30, 3.0]
    return x, v


def test_double_product_to_float_is_bit_exact(ctx):
    rng = np.random.default_rng(7)
    x, v = inputs(rng, 20000)
    for d in multipliers():
        mul, _ = ctx.selftest_conversions(x, d, v)
        want = (x.astype(np.float64) * np.float64(d)).astype(np.float32)
        bad = np.flatnonzero(mul.view(np.uint32) != want.view(np.uint32))
        assert bad.size == 0, (d, x[bad[:5]], mul[bad[:5]], want[bad[:5]])


def test_fixed_point_of_float_is_bit_exact(ctx):
    rng = np.random.default_rng(8)
    x, v = inputs(rng, 20000)
    _, fix = ctx.selftest_conversions(x, 1.0, v)
    want = np.rint(v.astype(np.float64) * 4294967296.0).astype(np.int64)
    bad = np.flatnonzero(fix != want)
    assert bad.size == 0, (v[bad[:5]], fix[bad[:5]], want[bad[:5]])
