"""bench.py's CPU side: the row-stratified tile samples and the --impl reference line.

The reference arm times the CPU oracle on a bounded sample of the config-2 frame. Nearly all
of that frame's CPU time sits in the terrain rows (a sky tile costs about a thousandth of a
terrain tile), so the sample takes one tile from each band of tile rows; a uniform draw of a
few tiles could land on sky only and overstate the rate many times over. The GPU arm's
CPU baseline takes two tiles from every tile row and reports a bootstrap interval.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

BW, BH = bench.W // 64, bench.H // 64


@pytest.mark.parametrize("n", [1, 3, 4, 16])
def test_tiles_are_one_per_band_of_rows(n):
    for seed in (0, 1, 1000):
        tiles = bench.cpu_tiles(n, seed)
        assert tiles == sorted(set(tiles)) and len(tiles) == n
        assert all(0 <= t < BW * BH for t in tiles)
        rows = [t // BW for t in tiles]
        for k, r in enumerate(rows):
            assert (k * BH) // n <= r < max((k * BH) // n + 1, ((k + 1) * BH) // n)
        assert bench.cpu_tiles(n, seed) == tiles   # seeded


def test_full_sample_takes_two_tiles_from_every_tile_row():
    rows = sorted(t // BW for t in bench.cpu_tiles(bench.CPU_SAMPLE_TILES, 0))
    assert rows == sorted(list(range(BH)) * 2)


def test_bootstrap_interval_brackets_the_measured_rate():
    """The CPU baseline's 95 % interval: tiles resampled within their row, scaled to the
    measured wall-clock rate; it contains that rate and widens with the spread of tile costs."""
    import numpy as np

    rng = np.random.default_rng(0)
    rows = np.repeat(np.arange(16), 2)
    rays = rng.integers(10_000, 20_000, size=32)
    even = rays / 1e5
    lo, hi = bench.bootstrap_rate(rays, even, rows, 0.25)
    assert lo == hi == 0.25   # every tile at the same rate: no spread
    uneven = even * rng.uniform(0.2, 5.0, size=32)
    lo, hi = bench.bootstrap_rate(rays, uneven, rows, 0.25)
    assert lo < 0.25 < hi


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], check=True, capture_output=True, text=True, timeout=600).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "Mrays/s"
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 3
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["cpu_model"]
    assert d["e2e"] == {"value": d["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
