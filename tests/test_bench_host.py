"""bench.py's roofline arithmetic on CPU: the per-kernel algorithmic bytes and
the whole-substep path roofline of the 1M-particle / 128^3 workload."""
from __future__ import annotations

import pytest

PEAK = {"hbm_gbs": 6779.7, "source": "measured"}


def test_path_bytes_are_the_six_dispatches():
    import bench
    # p2g_1 60 + p2g_2 48 + g2p 12 + 60 + copyPosition 24 per particle;
    # clear 16 + p2g_1 16 + p2g_2 28 + updateGrid 28 + g2p 12 per cell
    assert bench.PATH_BYTES_PER_PARTICLE == 204
    assert bench.PATH_BYTES_PER_CELL == 100
    r = bench.path_roofline(1_000_000, 128 ** 3, 1e10, PEAK)
    assert r["bytes_per_substep"] == 204 * 1_000_000 + 100 * 2_097_152  # 413.7 MB
    # 1e10 particle-substeps/s = 1e4 substeps/s x 413.7 MB = 4.14 TB/s
    assert r["achieved"] == pytest.approx(4137.152, rel=1e-9)
    assert r["frac"] == pytest.approx(0.6102, abs=1e-4)
    assert r["peak_source"] == "measured"


def test_path_roofline_scales_with_the_rate():
    import bench
    a = bench.path_roofline(64_000, 64 ** 3, 1e9, PEAK)
    b = bench.path_roofline(64_000, 64 ** 3, 2e9, PEAK)
    assert b["achieved"] == pytest.approx(2 * a["achieved"], rel=1e-12)
    # 64k particles on 64^3: 13.06 + 26.21 MB per substep
    assert a["bytes_per_substep"] == 204 * 64_000 + 100 * 262_144


def test_kernel_algorithmic_bytes():
    import bench
    n, cells = 1_000_000, 372_163
    # g2p in 12 + out 60 + half of the 24-byte posvel per substep; 32 per cell
    assert bench.algorithmic_bytes("sorted_g2p_p2g_1", n, cells) == n * 84 + cells * 32
    assert bench.algorithmic_bytes("sorted_p2g_2", n, cells) == n * 48 + cells * 28
    assert bench.algorithmic_bytes("updateGrid", n, cells) is None
