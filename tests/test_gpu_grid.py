"""GPU test of the uniform-grid sampler (UniformGrid, src/marching.cpp): the
lattice (dims, box) equals the oracle's restatement bit for bit, the values
are within the field tolerances of the FP64 and float oracles, and the VTK
image file holds exactly the sampled values."""
import re

import numpy as np
import pytest

import parity as PR
import pyoracle as O
from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B
from particleisosurface_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = {
    "blob2k": lambda: synth.small_blob(n=2000, seed=3),
    "slab_sphere_20k": lambda: synth.slab_and_sphere(n=20000, seed=1),
}


@pytest.fixture(scope="module")
def ctx():
    B.build()
    O.build()
    c = N.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", list(CASES))
def test_grid_matches_oracle(ctx, name, tmp_path):
    fr = CASES[name]()
    g = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz)
    g.hashgrid().aniso().normals()
    o = O.OracleFrame(fr.xyz, fr.radius)
    o64 = O.OracleFrame(fr.xyz, fr.radius, flags=O.FP64)
    for s in (1, 2, 3):
        o.stage(s)
        o64.stage(s)
    box_o, steps_o, dims_o = o.uniform_grid()
    dims_g, box_g, n = g.grid_dims()
    np.testing.assert_array_equal(dims_g, dims_o)
    np.testing.assert_array_equal(box_g, box_o)
    vg = g.grid_sample()
    vo = o.grid_sample()
    v64 = o64.grid_sample()
    ms = o.scalars()["max_scalar"]
    e_gpu = np.abs(vg - v64) / ms
    print(name, "grid", tuple(dims_g), "points", n, "err vs FP64 max %.3e rms %.3e | float oracle max %.3e"
          % (e_gpu.max(), np.sqrt(np.mean(e_gpu ** 2)), (np.abs(vo - v64) / ms).max()))
    assert e_gpu.max() <= PR.FIELD_TOL_FP64
    assert np.all(np.abs(vg - vo) <= np.maximum(PR.FIELD_TOL * ms, np.abs(vo - v64) + PR.FIELD_TOL_FP64 * ms))
    # the VTK image holds the same values
    path = tmp_path / "grid.vti"
    g.write_vti(str(path))
    raw = path.read_bytes()
    head = raw[:raw.index(b"<AppendedData")].decode()
    assert 'WholeExtent="0 %d 0 %d 0 %d"' % tuple(int(d) - 1 for d in dims_g) in head
    spacing = [float(x) for x in re.search(r'Spacing="([^"]+)"', head).group(1).split()]
    assert spacing == pytest.approx([fr.radius] * 3, rel=1e-6)
    start = raw.index(b"_", raw.index(b"<AppendedData")) + 1
    nbytes = int.from_bytes(raw[start:start + 8], "little")
    assert nbytes == 4 * n
    vals = np.frombuffer(raw[start + 8:start + 8 + nbytes], dtype="<f4")
    np.testing.assert_array_equal(vals, vg.ravel())
    g.close()
