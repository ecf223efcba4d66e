"""GPU parity of the variable-radius path (pi_frame_upload_radii) against the
oracle's variable-radius restatement (the reference's MultiLevelSearcher,
per-particle kernel constants and resizeRootBoxVarR with the neighbour query
switched on; src/multi_level_reseacher.cpp, src/evaluator.cpp:16-29,
src/surface_reconstructor.cpp:124-222), on two-radius frames (slab of radius
r under a sphere of radius 2r):

  bit-exact: the radius bins' grids (bounding box, cells, cell size, radius
  particle), every particle's grid and key, IndexList per grid, neighbour
  lists (GetNeighbors), iso value, MaxScalar, root and depths;
  within the tolerances of tests/parity.py: smoothed centres, G,
  determinants, normals and field values (the field also against the
  oracle's FP64 mode); octree node set and types identical except near the
  isovalue or a curvature of 0.99; mesh as in the constant-radius tests.
"""
import numpy as np
import pytest

import parity as PR
import pyoracle as O
from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B
from particleisosurface_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = {
    "two_radius_4k": lambda: synth.two_radius_frame(n=4000, seed=6),
    "two_radius_20k": lambda: synth.two_radius_frame(n=20000, seed=8),
}


@pytest.fixture(scope="module")
def ctx():
    B.build()
    O.build()
    c = N.Context(0)
    yield c
    c.close()


_cache = {}


def run_pair(ctx, name):
    if name not in _cache:
        fr = CASES[name]()
        o = O.OracleFrame(fr.xyz, fr.radii).run()
        o.frame_counts = (o.counter(0), o.counter(3))
        g = N.Frame(ctx, N.default_params(float(fr.radii.min()))).upload(fr.xyz).upload_radii(fr.radii).run()
        o64 = O.OracleFrame(fr.xyz, fr.radii, flags=O.FP64)
        for s in (1, 2, 3):
            o64.stage(s)
        _cache[name] = (fr, o, g, o64)
    return _cache[name]


@pytest.mark.parametrize("name", list(CASES))
def test_varr_grids_keys_and_lists_bit_exact(ctx, name):
    fr, o, g, _ = run_pair(ctx, name)
    bins = o.bins()
    info = g.info()
    assert info["num_grids"] == len(bins) >= 2
    sr = o.searcher_radii()
    assert info["radius_min"] == np.float32(sr["min"]) and info["radius_max"] == np.float32(sr["max"])
    keys = np.full(fr.n, -2, np.int64)
    grid_of = np.full(fr.n, -1, np.int32)
    for k, b in enumerate(bins):
        gk = g.grid(k)
        np.testing.assert_array_equal(gk["bounding"], b["bounding"])
        np.testing.assert_array_equal(gk["dims"], b["xyz_cell_num"])
        assert gk["cell_size"] == np.float32(b["cell_size"])
        assert gk["radius_id"] == b["radius_id"] and gk["count"] == len(b["particles"])
        keys[b["particles"]] = b["keys"]
        grid_of[b["particles"]] = k
    np.testing.assert_array_equal(g.dump(N.DUMP_KEYS), keys)
    np.testing.assert_array_equal(g.dump(N.DUMP_GRID_OF), grid_of)
    np.testing.assert_array_equal(g.dump(N.DUMP_INDEX_LIST), np.concatenate([b["index_list"] for b in bins]))
    rng = np.random.default_rng(1)
    lo, hi = fr.xyz.min(0), fr.xyz.max(0)
    pts = np.concatenate([fr.xyz[rng.choice(fr.n, 200)],
                          rng.uniform(lo - 0.05, hi + 0.05, size=(200, 3)).astype(np.float32)])
    off_o, idx_o = o.neighbors(pts)
    off_g, idx_g = g.neighbors(pts)
    np.testing.assert_array_equal(off_g, off_o)
    np.testing.assert_array_equal(idx_g, idx_o)


@pytest.mark.parametrize("name", list(CASES))
def test_varr_scalars_and_root_exact(ctx, name):
    fr, o, g, _ = run_pair(ctx, name)
    sc, d, info = o.scalars(), o.depths(), g.info()
    assert info["iso_value"] == np.float32(sc["iso"])
    assert info["max_scalar"] == np.float32(sc["max_scalar"])
    assert info["depth_max"] == d["depth_max"] and info["depth_min"] == d["depth_min"]
    np.testing.assert_array_equal(np.array(info["root_center"], np.float32), d["root_center"])
    assert info["root_half"] == np.float32(d["root_half"])


@pytest.mark.parametrize("name", list(CASES))
def test_varr_aniso_normals_field(ctx, name):
    fr, o, g, o64 = run_pair(ctx, name)
    r_min = float(fr.radii.min())
    xm, G, det = o.aniso()
    x64, G64, d64 = o64.aniso()
    gx, gG, gd = g.dump(N.DUMP_XMEANS), g.dump(N.DUMP_G), g.dump(N.DUMP_DET)
    assert np.abs(gx - x64).max() <= PR.XMEAN_TOL * r_min
    assert np.all(np.abs(gx - xm) <= np.abs(xm - x64) + PR.XMEAN_TOL * r_min)
    assert np.abs(gG - G64).max() <= PR.G_TOL and np.abs(gd - d64).max() <= PR.G_TOL
    assert np.all(np.abs(gG - G) <= np.abs(G - G64) + PR.G_TOL)
    no, n64 = o.normals(), o64.normals()
    scale = np.abs(n64).max()
    gn = g.dump(N.DUMP_NORMALS)
    assert np.abs(gn - n64).max() <= PR.NORMAL_TOL * scale
    assert np.all(np.abs(gn - no) <= np.abs(no - n64) + PR.NORMAL_TOL * scale)
    rng = np.random.default_rng(2)
    rad = fr.radii[rng.choice(fr.n, 2000)][:, None]
    pts = (fr.xyz[rng.choice(fr.n, 2000)] + rng.normal(0, 1.5, (2000, 3)) * rad).astype(np.float32)
    ms = o.scalars()["max_scalar"]
    sg, so, s64 = g.eval(pts).astype(np.float64), o.eval(pts), o64.eval(pts)
    e = np.abs(sg - s64) / ms
    print(name, "variable radius: field vs FP64 max %.3e rms %.3e (x MaxScalar), float reference %.3e"
          % (e.max(), np.sqrt(np.mean(e ** 2)), (np.abs(so - s64) / ms).max()))
    assert e.max() <= PR.FIELD_TOL_FP64
    assert np.all(np.abs(sg - so) <= np.maximum(PR.FIELD_TOL * ms, np.abs(so - s64) + PR.FIELD_TOL_FP64 * ms))


@pytest.mark.parametrize("name", list(CASES))
def test_varr_octree_and_mesh(ctx, name):
    fr, o, g, o64 = run_pair(ctx, name)
    ms = o.scalars()["max_scalar"]
    rep = PR.compare_octrees_fast(o.nodes(), g.dump(N.DUMP_NODES), o, ms, o.depths()["depth_min"],
                                  fp64_eval=o64.eval)
    print(name, {k: v for k, v in rep.items() if k != "unexplained"}, rep["unexplained"][:5])
    assert not rep["unexplained"]
    assert rep["explained"] <= max(2, rep["compared"] // 10000)
    assert rep["leaf_far_vs_fp64_max"] <= PR.FIELD_TOL_FP64
    nodes = g.dump(N.DUMP_NODES)
    leaf_depths = np.unique(nodes["depth"][nodes["type"] == 2])
    assert len(leaf_depths) >= 2, leaf_depths
    info = g.info()
    if rep["explained"] == 0:
        assert info["field_evals"] - info["bisection_evals"] == o.frame_counts[0] - o.frame_counts[1]
    m = PR.compare_meshes_fast(o.mesh(), g.mesh(keys=True), float(fr.radii.min()))
    print(name, {k: v for k, v in m.items() if k != "off_gpu_idx"})
    n_v = m["verts_oracle"]
    assert n_v > 0
    assert m["verts_only_oracle"] + m["verts_only_gpu"] <= max(4, n_v // 2000)
    assert m["tris_only_oracle"] + m["tris_only_gpu"] <= max(8, m["tris_oracle"] // 1000)
    assert m["verts_off_tol"] <= max(4, n_v // 2000)


def test_varr_equal_radii_equal_constant_radius_field(ctx):
    """Every radius equal: one grid, the constant-radius grid, and the same
    per-particle records, so the hash grid and the anisotropy equal the
    constant-radius path's bit for bit, and so does the field sum; the field
    values differ by the iso values alone (RecommendIsoValueVarR takes the
    kernel at ratio 0.25, RecommendIsoValueConstR at 0.01,
    src/evaluator.cpp:323-361)."""
    fr = synth.small_blob(n=3000, seed=12)
    gc = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
    gv = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).upload_radii(
        np.full(fr.n, fr.radius, np.float32)).run()
    assert gv.info()["num_grids"] == 1
    for what in (N.DUMP_KEYS, N.DUMP_INDEX_LIST, N.DUMP_XMEANS, N.DUMP_G, N.DUMP_DET):
        np.testing.assert_array_equal(gv.dump(what), gc.dump(what))
    pts = fr.xyz[::5] + np.float32(0.3 * fr.radius)
    iv, ic = gv.info()["iso_value"], gc.info()["iso_value"]
    assert iv < ic  # the kernel decreases: B(0.25) < B(0.01)
    ev, ec = gv.eval(pts).astype(np.float64), gc.eval(pts).astype(np.float64)
    # each value is iso - sum rounded to float: the sums agree to that rounding
    assert np.all(np.abs((iv - ev) - (ic - ec)) <= 2 * np.spacing(np.abs(ev).astype(np.float32)).astype(np.float64)
                  + 2 * np.spacing(np.float32(iv)))
    gc.close()
    gv.close()


def test_varr_rejects_bad_radii(ctx):
    fr = synth.small_blob(n=500, seed=13)
    f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz)
    with pytest.raises(N.PiError) as e:
        f.upload_radii(np.full(fr.n - 1, fr.radius, np.float32))
    assert e.value.code == N.PI_ERR_INVALID
    bad = np.full(fr.n, fr.radius, np.float32)
    bad[7] = -1.0
    with pytest.raises(N.PiError) as e:
        f.upload_radii(bad)
    assert e.value.code == N.PI_ERR_INVALID
    f.close()
    fq = N.Frame(ctx, N.default_params(fr.radius, qef=True)).upload(fr.xyz)
    with pytest.raises(N.PiError) as e:
        fq.upload_radii(np.full(fr.n, fr.radius, np.float32))
    assert e.value.code == N.PI_ERR_INVALID
    fq.close()
