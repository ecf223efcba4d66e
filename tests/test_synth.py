"""CPU tests of the seeded synthetic workloads (no GPU): each generator is a
pure function of its seed (two calls give the same particles bit for bit, a
different seed gives others), returns the particle count asked for, and the
1M dam-break frame has the geometry scale the measurements quote."""
import numpy as np
import pytest

from particleisosurface_gb300 import synth

GENERATORS = {
    "slab_and_sphere": lambda seed: synth.slab_and_sphere(n=20000, seed=seed),
    "small_blob": lambda seed: synth.small_blob(n=2000, seed=seed),
    "spray_frame": lambda seed: synth.spray_frame(n=6000, seed=seed),
    "sheets_and_filaments": lambda seed: synth.sheets_and_filaments(n=50_000, seed=seed),
    "mixed_frame": lambda seed: synth.mixed_frame(seed, 60_000),
}


@pytest.mark.parametrize("name", list(GENERATORS))
def test_generator_is_a_function_of_its_seed(name):
    a, b, c = GENERATORS[name](11), GENERATORS[name](11), GENERATORS[name](12)
    assert a.xyz64.shape == b.xyz64.shape and np.array_equal(a.xyz64, b.xyz64)
    assert a.xyz64.shape != c.xyz64.shape or not np.array_equal(a.xyz64, c.xyz64)
    assert np.all(np.isfinite(a.xyz64)) and a.radius > 0


@pytest.mark.parametrize("name,n", [("slab_and_sphere", 20000), ("small_blob", 2000), ("spray_frame", 6000)])
def test_generator_returns_the_count_asked_for(name, n):
    assert GENERATORS[name](5).n == n


def test_dam_break_frame_of_the_measurements():
    fr = synth.dam_break(n=1_000_000, seed=2)
    assert fr.n == 1_000_000 and fr.radius == pytest.approx(0.01)
    assert fr.scale == pytest.approx(3.778, abs=5e-4)
    again = synth.dam_break(n=1_000_000, seed=2)
    assert np.array_equal(fr.xyz, again.xyz)
