"""Host-side helpers of bench.py that turn measurements into the JSON line: the batched
row-pass roofline parsed from the autotuner's report."""

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    pytest.importorskip("torch")
    sys.path.insert(0, str(ROOT))
    import bench

    return bench


def test_batched_row_roofline_from_tuning_report():
    bench = _bench()
    tune = {
        64: ["fp32 row flags=14 batched D=3 grid=64x64x1 solves=176 -> v0=30.0us v4=28.0us chosen v4"],
        256: ["fp32 x n=256 lines=135168 mode=0 D=3 grid=256x256x1 solves=176 -> v0=250.0us chosen v0",
              "fp32 row flags=14 batched D=3 grid=256x256x1 solves=176 -> v0=569.343us v4=514.4us chosen v4",
              "row variant 4"],
    }
    r = bench.batched_row_roofline(tune)
    n_bytes = 176 * 2 * 3 * 65536 * 8 + 65536 * 4
    assert r["bytes_per_launch"] == n_bytes
    assert r["us_per_launch"] == pytest.approx(514.4)
    assert r["achieved"] == pytest.approx(n_bytes / 514.4e-6 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert "variant 4" in r["kernel"] and r["unit"] == "GB/s" and r["bound"] == "hbm"


def test_batched_row_roofline_absent_line():
    bench = _bench()
    assert bench.batched_row_roofline({256: ["row variant 0"]}) is None
