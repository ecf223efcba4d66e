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


def test_reciprocal_cell_index_agrees_with_division_where_trusted():
    """The sample bucketing's cell index (csrc/device.cuh, cell_coord_q):
    where fl(d * fl(1 / cell)) lies farther than 1e-6 * max(1, |q|) from
    every integer it truncates to the cell of the IEEE quotient fl(d / cell)
    (HashGrid::CalcXYZIdx); elsewhere the division is used.  Checked on
    random offsets and on offsets placed next to cell boundaries."""
    rng = np.random.default_rng(3)
    n = 2_000_000
    cell = (rng.uniform(0.5, 2.0, n) * 10.0 ** rng.integers(-4, 2, n)).astype(np.float32)
    k = rng.integers(-3, 4000, n).astype(np.float64)
    # offsets at random places and within a few ulps of a cell boundary
    frac = np.where(rng.random(n) < 0.5, rng.random(n), rng.choice([-1, 1], n) * rng.random(n) * 1e-6)
    d = ((k + frac) * cell.astype(np.float64)).astype(np.float32)
    rcell = (np.float32(1.0) / cell).astype(np.float32)
    with np.errstate(all="ignore"):
        q = (d * rcell).astype(np.float32)
        exact = (d / cell).astype(np.float32)
    dist = np.abs(q - np.rint(q))
    trusted = dist > np.float32(1e-6) * np.maximum(np.float32(1.0), np.abs(q))
    assert trusted.mean() > 0.4 and (~trusted).sum() > 1000
    np.testing.assert_array_equal(np.trunc(q[trusted]), np.trunc(exact[trusted]))
