"""The float forms of the reference's float-against-double comparisons
(particleisosurface_gb300/csrc/common.cuh): each constant must be the float
next to its double literal, so that one float comparison decides exactly as
the reference's promoted comparison (src/surface_reconstructor.cpp:247,262,
src/visitorextract.cpp:71-80)."""
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.path.dirname(HERE), "particleisosurface_gb300", "csrc", "common.cuh")


def _const(name):
    text = open(SRC).read()
    m = re.search(r"constexpr float %s = (0x[0-9a-fA-F.]+p[-+]?\d+)f;" % name, text)
    assert m, name
    return np.float32(float.fromhex(m.group(1)))


def test_thresholds_are_the_floats_next_to_the_literals():
    inf = np.float32(np.inf)
    for name, d in (("kAbove1em8", 1e-8), ("kAbove099", 0.99), ("kAbove01", 0.1)):
        c = _const(name)
        assert float(c) > d and float(np.nextafter(c, -inf)) < d, name
    c = _const("kBelow09")
    assert float(c) < 0.9 and float(np.nextafter(c, inf)) > 0.9


def test_float_comparison_equals_promoted_comparison():
    rng = np.random.default_rng(0)
    for name, d, op in (("kAbove1em8", 1e-8, "lt"), ("kAbove099", 0.99, "lt"), ("kAbove01", 0.1, "lt"),
                        ("kBelow09", 0.9, "gt")):
        c = _const(name)
        # every float within 64 ulps of the literal, and random ones around it
        base = np.float32(d)
        xs = [base]
        for _ in range(64):
            xs.append(np.nextafter(xs[-1], np.float32(np.inf)))
        x = base
        for _ in range(64):
            x = np.nextafter(x, np.float32(-np.inf))
            xs.append(x)
        xs = np.concatenate([np.array(xs, np.float32),
                             (d * rng.uniform(0.5, 1.5, 10000)).astype(np.float32)])
        if op == "lt":
            np.testing.assert_array_equal(xs < c, xs.astype(np.float64) < d)
        else:
            np.testing.assert_array_equal(xs > c, xs.astype(np.float64) > d)
