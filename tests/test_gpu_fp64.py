"""GPU test of the FP64 oracle (pi_fp64_aniso / pi_fp64_eval_field /
pi_fp64_scalars) against the CPU oracle's FP64 mode (oracle/pi_oracle.cpp
with PIO_FP64): the same formulas (src/evaluator.cpp:60-125,465-654) in
double on the same float inputs and hash grid, so they agree to double
rounding.  The bounds below are far under the FP32 path's tolerances
(tests/parity.py), which these values arbitrate.
"""
import numpy as np
import pytest

import pyoracle as O
from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B
from particleisosurface_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = {
    "slab_sphere_20k": lambda: synth.slab_and_sphere(n=20000, seed=1),
    "sheets_20k": lambda: synth.sheets_and_filaments(n=20000, seed=9),
    "blob2k": lambda: synth.small_blob(n=2000, seed=3),
}


@pytest.fixture(scope="module")
def ctx():
    B.build()
    O.build()
    c = N.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", list(CASES))
def test_fp64_oracle_matches_cpu_fp64(ctx, name):
    fr = CASES[name]()
    g = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).hashgrid()
    o = O.OracleFrame(fr.xyz, fr.radius, flags=O.FP64)
    for s in (1, 2, 3):
        o.stage(s)
    sc, so = g.scalars_fp64(), o.scalars()
    for k in ("iso", "max_scalar", "influence2", "sigma"):
        assert sc[k] == pytest.approx(so[k], rel=1e-14), k
    x64, G64, d64 = g.aniso_fp64()
    xo, Go, do = o.aniso()
    ex = np.abs(x64 - xo).max()
    eG = np.abs(G64 - Go).max()
    ed = np.abs(d64 - do).max()
    rng = np.random.default_rng(5)
    pts = (fr.xyz[rng.choice(fr.n, 3000)] + rng.normal(0, 1.5 * fr.radius, (3000, 3))).astype(np.float32)
    v64, g64 = g.eval_fp64(pts, grad=True)
    vo, go = o.eval(pts, grad=True)
    ev = np.abs(v64 - vo).max() / so["max_scalar"]
    eg = np.abs(g64 - go).max() / max(np.abs(go).max(), 1e-300)
    print(name, "FP64 GPU vs FP64 CPU: centres %.2e, G %.2e, det %.2e, field %.2e (x MaxScalar), grad %.2e (rel)"
          % (ex, eG, ed, ev, eg))
    assert ex <= 1e-12 and eG <= 1e-9 and ed <= 1e-9
    assert ev <= 1e-10 and eg <= 1e-9
    # the state follows the frame: a reset and a second run recompute it
    g.reset().hashgrid()
    v2 = g.eval_fp64(pts)
    np.testing.assert_array_equal(v2, v64)
    g.close()


def test_fp64_needs_hash_grid(ctx):
    fr = synth.small_blob(n=500, seed=4)
    g = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz)
    with pytest.raises(N.PiError) as e:
        g.eval_fp64(fr.xyz[:4])
    assert e.value.code == N.PI_ERR_STATE
    g.close()
