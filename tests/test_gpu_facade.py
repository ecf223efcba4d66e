"""GPU test of the C++ facade: a host program using the reference's class
names (SurfReconstructor::Run, Evaluator, HashGrid, TNode, writeObjFile)
produces the same OBJ file, byte for byte, as the library's own writer on the
same particles, and its queries agree with the oracle."""
import json
import subprocess

import numpy as np
import pytest

import facade
from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import synth

pytestmark = pytest.mark.gpu


def test_facade_obj_identical_to_library_writer(tmp_path):
    import pyoracle as O
    exe = facade.build()
    fr = synth.small_blob(n=2500, seed=11)
    src = tmp_path / "xyz.f32"
    fr.xyz.astype(np.float32).tofile(src)
    r = subprocess.run([exe, str(src), str(fr.n), repr(fr.radius), str(tmp_path / "facade.obj")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])

    ctx = N.Context(0)
    f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
    f.write_obj(str(tmp_path / "lib.obj"))
    info = f.info()
    assert (tmp_path / "facade.obj").read_bytes() == (tmp_path / "lib.obj").read_bytes()
    f.write_ply(str(tmp_path / "lib.ply"))
    assert (tmp_path / "facade.obj.ply").read_bytes() == (tmp_path / "lib.ply").read_bytes()
    # the same particles through loadParticlesFromCSV give the same mesh
    csv = tmp_path / "p.csv"
    csv.write_text('"Points:0","Points:1","Points:2"\n' + "\n".join("%.9g,%.9g,%.9g" % tuple(p) for p in fr.xyz) + "\n")
    r2 = subprocess.run([exe, str(csv), "0", repr(fr.radius), str(tmp_path / "csv.obj")],
                        capture_output=True, text=True, timeout=300)
    assert r2.returncode == 0, r2.stdout + r2.stderr
    assert (tmp_path / "csv.obj").read_bytes() == (tmp_path / "lib.obj").read_bytes()
    f.close()
    # UniformGrid through the facade writes the library's VTK image
    fg = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz)
    fg.hashgrid().aniso().normals()
    fg.write_vti(str(tmp_path / "lib_grid.vti"))
    dims, _, npts = fg.grid_dims()
    fg.close()
    ctx.close()
    assert (tmp_path / "grid.vti").read_bytes() == (tmp_path / "lib_grid.vti").read_bytes()
    assert out["grid_dims"] == [int(d) for d in dims] and out["grid_points"] == npts
    assert out["vertices"] == info["num_vertices"] and out["triangles"] == info["num_triangles"]
    assert out["depth_max"] == info["depth_max"] and out["nodes"] == info["num_nodes"]

    o = O.OracleFrame(fr.xyz, fr.radius)
    for s in (1, 2, 3):
        o.stage(s)
    sc = o.scalars()
    assert out["iso"] == pytest.approx(sc["iso"], rel=1e-6)
    assert out["max_scalar"] == pytest.approx(sc["max_scalar"], rel=1e-6)
    off, idx = o.neighbors(fr.xyz[:1])
    assert out["neighbors0"] == len(idx)
    assert out["key0"] == int(o.keys()[0])
    assert abs(out["scalar0"] - float(o.eval(fr.xyz[:1])[0])) <= 3e-5 * sc["max_scalar"]


def test_facade_variable_radius_equals_library(tmp_path):
    """IS_CONST_RADIUS false in the host program: SurfReconstructor takes the
    per-particle radii (pi_frame_upload_radii), the mesh equals the
    library's, and getSearcher() reports the searcher's radii and bins."""
    exe = facade.build()
    fr = synth.two_radius_frame(n=4000, seed=6)
    src, rad = tmp_path / "xyz.f32", tmp_path / "r.f32"
    fr.xyz.astype(np.float32).tofile(src)
    fr.radii.astype(np.float32).tofile(rad)
    r = subprocess.run([exe, str(src), str(fr.n), "0.5", str(tmp_path / "facade.obj"), str(rad)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    ctx = N.Context(0)
    f = N.Frame(ctx, N.default_params(float(fr.radii.min()))).upload(fr.xyz).upload_radii(fr.radii).run()
    f.write_obj(str(tmp_path / "lib.obj"))
    assert (tmp_path / "facade.obj").read_bytes() == (tmp_path / "lib.obj").read_bytes()
    info = f.info()
    assert out["grids"] == info["num_grids"] >= 2 and out["has_hash_grid"] == 0
    assert out["min_radius"] == pytest.approx(info["radius_min"], rel=1e-7)
    assert out["max_radius"] == pytest.approx(info["radius_max"], rel=1e-7)
    assert out["depth_max"] == info["depth_max"] and out["vertices"] == info["num_vertices"]
    off, idx = f.neighbors(fr.xyz[:1])
    assert out["neighbors0"] == len(idx)
    f.close()
    ctx.close()


def test_facade_hdf5_input_equals_array_input(tmp_path):
    """readShonDyParticleData through the facade: an HDF5 particle file
    (flat "position" of doubles) gives the mesh of the same particles
    passed as floats."""
    import h5write as W
    exe = facade.build()
    fr = synth.small_blob(n=2500, seed=11)
    W.write_particles(tmp_path / "p.h5", fr.xyz64, layout="v0", storage="chunked", chunk=1000,
                      filters=("shuffle", "deflate"))
    r = subprocess.run([exe, str(tmp_path / "p.h5"), "0", repr(fr.radius), str(tmp_path / "h5.obj")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ctx = N.Context(0)
    f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
    f.write_obj(str(tmp_path / "lib.obj"))
    f.close()
    ctx.close()
    assert (tmp_path / "h5.obj").read_bytes() == (tmp_path / "lib.obj").read_bytes()
