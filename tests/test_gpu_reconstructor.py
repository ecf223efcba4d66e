"""GPU test of the Python facade with the reference's class names
(particleisosurface_gb300/reconstructor.py): SurfReconstructor.Run, Mesh,
writeObjFile, HashGrid, Evaluator and UniformGrid give what the C ABI gives
for the same frame, and the hash-grid queries what the oracle gives.
Mirrors a caller of src/surface_reconstructor.cpp:409 and src/main.cpp:54-67.
"""
import numpy as np
import pytest

import pyoracle as O
from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B
from particleisosurface_gb300 import reconstructor as R
from particleisosurface_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    B.build()
    O.build()
    c = N.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("qef", [False, True])
def test_surf_reconstructor_run_equals_pi_run(ctx, qef, tmp_path):
    fr = synth.slab_and_sphere(n=6000, seed=41)
    mesh = R.Mesh()
    rec = R.SurfReconstructor(fr.xyz, np.zeros(0, np.float32), mesh, fr.radius, ctx=ctx, qef=qef)
    rec.Run(1.9, 2.0)
    g = N.Frame(ctx, N.default_params(fr.radius, qef=qef)).upload(fr.xyz).run()
    v, t, k = g.mesh(keys=True)
    np.testing.assert_array_equal(mesh.vertices, v)
    np.testing.assert_array_equal(mesh.tris, t + 1)  # 1-based, as Mesh::tris
    np.testing.assert_array_equal(mesh.vertex_keys, k)
    assert mesh.verticesNum == len(v) and mesh.trianglesNum == len(t) and len(t) > 0
    # getters (include/surface_reconstructor.h:81-92)
    info = g.info()
    assert rec.getDepthMax() == info["depth_max"] and rec.getDepthMin() == info["depth_min"]
    assert rec.getGlobalParticlesNum() == fr.n and rec.getConstRadius() == pytest.approx(fr.radius)
    nodes = rec.getRoot()
    assert len(nodes) == info["num_nodes"] and int(nodes[0]["parent"]) == -1
    # writeObjFile: the same bytes as the library's OBJ writer
    a, b = tmp_path / "facade.obj", tmp_path / "lib.obj"
    R.writeObjFile(mesh, str(a))
    g.write_obj(str(b))
    assert a.read_bytes() == b.read_bytes()
    g.close()


def test_hashgrid_and_evaluator_facades(ctx):
    fr = synth.small_blob(n=3000, seed=42)
    mesh = R.Mesh()
    rec = R.SurfReconstructor(fr.xyz, np.zeros(0, np.float32), mesh, fr.radius, ctx=ctx)
    rec.Run()
    o = O.OracleFrame(fr.xyz, fr.radius)
    for s in (1, 2, 3):
        o.stage(s)
    hg = rec.getHashGrid()
    gi = o.grid_info()
    np.testing.assert_array_equal(hg.Bounding, gi["bounding"])
    assert hg.CellNum == gi["cell_num"]
    np.testing.assert_array_equal(hg.IndexList, o.index_list())
    rng = np.random.default_rng(4)
    for p in fr.xyz[rng.choice(fr.n, 20)]:
        off, idx = o.neighbors(p.reshape(1, 3))
        assert hg.GetPIdxList(p) == idx.tolist()
        h = np.float32(2 * fr.radius)
        assert hg.GetInBoxParticles(p - h, p + h) == o.in_box(p - h, p + h).tolist()
    ev = rec.getEvaluator()
    pts = fr.xyz[rng.choice(fr.n, 50)] + np.float32(0.5 * fr.radius)
    g = rec._frame
    want_s, want_g = g.eval(pts, grad=True)
    for k, p in enumerate(pts):
        s = ev.SingleEval(p)
        s2, gr = ev.SingleEvalWithGrad(p)
        assert s == want_s[k] and s2 == want_s[k]
        np.testing.assert_array_equal(gr, want_g[k])
    assert ev.getIsoValue() == g.info()["iso_value"]
    np.testing.assert_array_equal(ev.GlobalGs, g.dump(N.DUMP_G))
    np.testing.assert_array_equal(ev.PariclesNormals, g.dump(N.DUMP_NORMALS))


def test_uniform_grid_facade(ctx, tmp_path):
    fr = synth.small_blob(n=2000, seed=43)
    ug = R.UniformGrid(fr.xyz, fr.radius, ctx=ctx)
    vals = ug.Run(filename="grid", filepath=str(tmp_path))
    f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz)
    f.hashgrid().aniso().normals()
    dims, box, npts = f.grid_dims()
    np.testing.assert_array_equal(ug.dims, dims)
    np.testing.assert_array_equal(vals, f.grid_sample().ravel())
    assert (tmp_path / "grid.vti").stat().st_size > 4 * npts
    f.close()


def test_surf_reconstructor_variable_radius(ctx):
    """IS_CONST_RADIUS = False: Run takes the per-particle radii, the mesh is
    pi_run's with pi_frame_upload_radii, and getSearcher() describes the
    radius bins; the radius argument is not used."""
    fr = synth.two_radius_frame(n=4000, seed=6)
    mesh = R.Mesh()
    rec = R.SurfReconstructor(fr.xyz, fr.radii, mesh, 123.0, ctx=ctx)
    R.IS_CONST_RADIUS = False
    try:
        rec.Run(1.9, 2.0)
    finally:
        R.IS_CONST_RADIUS = True
    g = N.Frame(ctx, N.default_params(float(fr.radii.min()))).upload(fr.xyz).upload_radii(fr.radii).run()
    v, t, k = g.mesh(keys=True)
    np.testing.assert_array_equal(mesh.vertices, v)
    np.testing.assert_array_equal(mesh.tris, t + 1)
    assert rec.getHashGrid() is None
    s = rec.getSearcher()
    info = g.info()
    assert s.getMinRadius() == info["radius_min"] and s.getMaxRadius() == info["radius_max"]
    assert len(s.getSearchers()) == info["num_grids"] >= 2
    assert sum(b["count"] for b in s.getSearchers()) == fr.n
    p = fr.xyz[17]
    off, idx = g.neighbors(p.reshape(1, 3))
    assert s.GetNeighbors(p) == idx.tolist()
    g.close()
