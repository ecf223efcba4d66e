"""CPU tests of bench.py's arithmetic and defaults (no GPU): the per-group
roofline (candidate pairs x 38 FP32 flops, QEF leaves x 960 FP64 flops,
over each group's own event time) and the command-line defaults the
benchmark contract depends on."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_roofline_groups_arithmetic():
    steps = 20
    groups = {
        "chunked_sampling": dict(ms=146.2, launches=340, pairs=2_859_009_569 * steps, units=60_198_126 * steps),
        "qef": dict(ms=165.1, launches=380, pairs=0, units=4_218_176 * steps),
        "leaf_values": dict(ms=0.0, launches=0, pairs=0, units=0),  # not run: left out
    }
    out = bench.roofline_groups(groups, steps, fp32_peak=70.0, fp64_peak=1.1)
    assert set(out) == {"chunked_sampling", "qef"}
    cs = out["chunked_sampling"]
    want = 2_859_009_569 * steps * bench.FLOPS_PER_PAIR / (146.2e-3) / 1e12
    assert cs["achieved"] == pytest.approx(want)
    assert cs["frac"] == pytest.approx(want / 70.0)
    assert (cs["bound"], cs["unit"]) == ("fp32", "TFLOP/s")
    assert cs["ms_per_step"] == pytest.approx(146.2 / steps) and cs["launches_per_step"] == 17
    assert cs["pairs_per_step"] == 2_859_009_569
    q = out["qef"]
    assert bench.QEF_FLOPS_PER_LEAF == 27 * 15 * 2 + 150
    wq = 4_218_176 * steps * bench.QEF_FLOPS_PER_LEAF / (165.1e-3) / 1e12
    assert q["achieved"] == pytest.approx(wq) and q["frac"] == pytest.approx(wq / 1.1)
    assert q["bound"] == "fp64" and q["units_per_step"] == 4_218_176


def test_cli_defaults(monkeypatch):
    """No flags: one GPU, a few minutes of work, the library's own tuning."""
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert (a.gpus, a.impl, a.workload, a.n) == (1, "ours", "dam_break_1m", 1_000_000)
    assert a.warmup >= 3 and 1 <= a.steps <= 50
    assert a.qef_parts == 0 and a.eval_config == -1 and a.samples_per_lane == 0
