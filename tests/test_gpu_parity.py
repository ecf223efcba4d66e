"""GPU parity: the CUDA library (through the C ABI) against the oracle on the
same seeded inputs, stage by stage.

Bit-exact: grid parameters, cell keys, IndexList (cell order), cell offsets,
GetPIdxList / GetInBoxParticles lists, iso/MaxScalar/Sigma/Influnce2, octree
root and depths.  Within the tolerances of tests/parity.py: smoothed centres,
G, determinants, normals, field values, leaf values, mesh vertices.  Octree
classification and mesh topology identical except where a sample lies within
ISO_EPS of the isovalue or a curvature within CURV_EPS of 0.99 (counted).
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
    "blob2k": lambda: synth.small_blob(n=2000, seed=3),
    "slab6k": lambda: synth.slab_and_sphere(n=6000, seed=7),
    # the CPU-runnable single frame: 20,000 particles on a slab and a sphere, r = 0.025
    "slab_sphere_20k": lambda: synth.slab_and_sphere(n=20000, seed=1),
    # the precision-stress geometry (thin sheets, filaments) at a parity size
    "sheets_20k": lambda: synth.sheets_and_filaments(n=20000, seed=9),
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
    if name in _cache:
        return _cache[name]
    fr = CASES[name]()
    o = O.OracleFrame(fr.xyz, fr.radius).run()
    g = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
    _cache[name] = (fr, o, g)
    return _cache[name]


_cache64 = {}


def fp64_oracle(name):
    if name not in _cache64:
        fr = CASES[name]()
        o64 = O.OracleFrame(fr.xyz, fr.radius, flags=O.FP64)
        for s in (1, 2, 3):
            o64.stage(s)
        _cache64[name] = o64
    return _cache64[name]


@pytest.mark.parametrize("name", list(CASES))
def test_hashgrid_bit_exact(ctx, name):
    fr, o, g = run_pair(ctx, name)
    gi = o.grid_info()
    info = g.info()
    np.testing.assert_array_equal(np.array(info["bounding"], np.float32), gi["bounding"])
    np.testing.assert_array_equal(info["xyz_cell_num"], gi["xyz_cell_num"])
    assert info["cell_num"] == gi["cell_num"]
    assert info["cell_size"] == np.float32(gi["cell_size"])
    np.testing.assert_array_equal(g.dump(N.DUMP_KEYS), o.keys())
    np.testing.assert_array_equal(g.dump(N.DUMP_INDEX_LIST), o.index_list())
    off = g.dump(N.DUMP_CELL_OFFSETS)
    h, s, e = o.cells()
    np.testing.assert_array_equal(off[h], s)
    np.testing.assert_array_equal(off[h + 1], e)
    occupied = np.zeros(gi["cell_num"], bool)
    occupied[h] = True
    assert np.all(off[:-1][~occupied] == off[1:][~occupied])


@pytest.mark.parametrize("name", list(CASES))
def test_neighbor_lists_bit_exact(ctx, name):
    fr, o, g = run_pair(ctx, name)
    rng = np.random.default_rng(1)
    b = o.grid_info()["bounding"]
    lo, hi = b[0::2], b[1::2]
    pts = np.concatenate([fr.xyz[rng.choice(fr.n, 200)],
                          rng.uniform(lo - 0.1, hi + 0.1, size=(200, 3)).astype(np.float32)])
    off_o, idx_o = o.neighbors(pts)
    off_g, idx_g = g.neighbors(pts)
    np.testing.assert_array_equal(off_g, off_o)
    np.testing.assert_array_equal(idx_g, idx_o)
    for k in range(5):
        c = fr.xyz[rng.integers(fr.n)]
        h = np.float32(fr.radius * (1 + 3 * k))
        np.testing.assert_array_equal(g.in_box(c - h, c + h), o.in_box(c - h, c + h))


@pytest.mark.parametrize("name", list(CASES))
def test_scalars_and_root_exact(ctx, name):
    fr, o, g = run_pair(ctx, name)
    sc = o.scalars()
    d = o.depths()
    info = g.info()
    assert info["iso_value"] == np.float32(sc["iso"])
    assert info["max_scalar"] == np.float32(sc["max_scalar"])
    assert info["sigma"] == np.float32(sc["sigma"])
    assert info["influence2"] == np.float32(sc["influence2"])
    assert info["depth_max"] == d["depth_max"] and info["depth_min"] == d["depth_min"]
    np.testing.assert_array_equal(np.array(info["root_center"], np.float32), d["root_center"])
    assert info["root_half"] == np.float32(d["root_half"])


@pytest.mark.parametrize("name", list(CASES))
def test_aniso_within_tolerance(ctx, name):
    fr, o, g = run_pair(ctx, name)
    xm, G, det = o.aniso()
    dx = np.abs(g.dump(N.DUMP_XMEANS) - xm).max()
    dG = np.abs(g.dump(N.DUMP_G) - G).max()
    dd = np.abs(g.dump(N.DUMP_DET) - det).max()
    assert dx <= PR.XMEAN_TOL * fr.radius, dx
    assert dG <= PR.G_TOL, dG
    assert dd <= PR.G_TOL, dd


@pytest.mark.parametrize("name", list(CASES))
def test_normals_within_tolerance(ctx, name):
    fr, o, g = run_pair(ctx, name)
    no = o.normals()
    ng = g.dump(N.DUMP_NORMALS)
    scale = np.abs(no).max()
    assert np.abs(ng - no).max() <= PR.NORMAL_TOL * scale


@pytest.mark.parametrize("name", list(CASES))
def test_field_and_gradient_within_tolerance(ctx, name):
    fr, o, g = run_pair(ctx, name)
    rng = np.random.default_rng(2)
    pts = (fr.xyz[rng.choice(fr.n, 2000)] + rng.normal(0, 1.5 * fr.radius, (2000, 3))).astype(np.float32)
    so, go = o.eval(pts, grad=True)
    sg, gg = g.eval(pts, grad=True)
    s64 = fp64_oracle(name).eval(pts)
    ms = o.scalars()["max_scalar"]
    e_gpu = np.abs(sg - s64) / ms
    e_ref = np.abs(so - s64) / ms
    print(name, "field err vs FP64: gpu max %.3e rms %.3e | float oracle max %.3e rms %.3e"
          % (e_gpu.max(), np.sqrt(np.mean(e_gpu ** 2)), e_ref.max(), np.sqrt(np.mean(e_ref ** 2))))
    assert e_gpu.max() <= PR.FIELD_TOL_FP64
    # against the float oracle: its own error against FP64 plus ours (on thin
    # sheets the reference's float SVD is ~1e-4 * MaxScalar off FP64)
    assert np.all(np.abs(sg - so) <= np.maximum(PR.FIELD_TOL * ms, np.abs(so - s64) + PR.FIELD_TOL_FP64 * ms))
    assert np.abs(gg - go).max() <= PR.NORMAL_TOL * max(np.abs(go).max(), 1e-30)


@pytest.mark.parametrize("name", list(CASES))
def test_octree_identical_except_near_iso(ctx, name):
    fr, o, g = run_pair(ctx, name)
    rep = PR.compare_octrees(o.nodes(), g.dump(N.DUMP_NODES), o, o.scalars()["max_scalar"],
                             o.depths()["depth_min"])
    print(name, {k: v for k, v in rep.items() if k not in ("unexplained", "leaf_far_pos", "leaf_far_gpu")},
          rep["unexplained"][:5])
    assert not rep["unexplained"]
    assert rep["explained"] <= max(2, rep["compared"] // 10000)
    if rep["explained"] == 0:
        # the library counts the SingleEval calls the reference makes for the
        # octree (the oracle's counter 0 minus its bisection calls)
        info = g.info()
        assert info["field_evals"] - info["bisection_evals"] == o.counter(0) - o.counter(3)
        assert 0 < info["field_evals_performed"] <= info["field_evals"]
    ms = o.scalars()["max_scalar"]
    if rep["leaf_value_maxdiff"] > PR.FIELD_TOL * ms:
        # leaves where the float oracle and the library differ by more than
        # FIELD_TOL: the library must then be within FIELD_TOL_FP64 of FP64
        pos, vg = rep["leaf_far_pos"], rep["leaf_far_gpu"]
        v64 = fp64_oracle(name).eval(pos)
        err = np.abs(vg - v64) / ms
        print(name, "%d leaves beyond FIELD_TOL of the float oracle; library vs FP64 max %.3e"
              % (len(pos), err.max()))
        assert err.max() <= PR.FIELD_TOL_FP64


@pytest.mark.parametrize("name", list(CASES))
def test_mesh_matches(ctx, name):
    fr, o, g = run_pair(ctx, name)
    rep = PR.compare_meshes_fast(o.mesh(), g.mesh(keys=True), fr.radius)
    print(name, {k: v for k, v in rep.items() if k != "off_gpu_idx"})
    assert rep["verts_oracle"] > 0
    n_v = rep["verts_oracle"]
    assert rep["verts_only_oracle"] + rep["verts_only_gpu"] <= max(4, n_v // 2000)
    assert rep["tris_only_oracle"] + rep["tris_only_gpu"] <= max(8, rep["tris_oracle"] // 1000)
    # vertices off the float oracle's: the FP64 bisection of the same edge decides
    agree, expl, bad = PR.check_vertices_fp64(g, rep, fr.radius, o.scalars()["max_scalar"], N.DUMP_NODES,
                                              N.DUMP_VERTEX_EDGES)
    print(name, "off tolerance %d: agree with FP64 %d, near tie %d" % (rep["verts_off_tol"], agree, expl))
    assert len(bad) == 0, bad[:10]
    assert expl <= max(4, n_v // 2000)


def test_reconstruct_host_roundtrip(ctx):
    fr = synth.small_blob(n=1500, seed=9)
    v, t = ctx.reconstruct(fr.xyz, N.default_params(fr.radius))
    g = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
    v2, t2 = g.mesh()
    np.testing.assert_array_equal(v, v2)
    np.testing.assert_array_equal(t, t2)


def test_reconstruct_reuses_its_frame(ctx):
    """pi_reconstruct keeps one frame per context (no budget): calls on
    different inputs and parameters in a row, a failed call among them, each
    give what a fresh frame gives."""
    a = synth.small_blob(n=1500, seed=9)
    b = synth.slab_and_sphere(n=6000, seed=7)

    def fresh(fr, qef=False):
        g = N.Frame(ctx, N.default_params(fr.radius, qef=qef)).upload(fr.xyz).run()
        m = g.mesh()
        g.close()
        return m

    want_a, want_b, want_bq = fresh(a), fresh(b), fresh(b, qef=True)
    bad = np.zeros((10, 3), np.float32)
    bad[3, 1] = np.nan
    for fr, params, want in ((a, N.default_params(a.radius), want_a),
                             (b, N.default_params(b.radius), want_b),
                             (bad, N.default_params(0.01), None),
                             (b, N.default_params(b.radius, qef=True), want_bq),
                             (a, N.default_params(a.radius), want_a)):
        if want is None:
            with pytest.raises(N.PiError):
                ctx.reconstruct(fr, params)
            continue
        v, t = ctx.reconstruct(fr.xyz, params)
        np.testing.assert_array_equal(v, want[0])
        np.testing.assert_array_equal(t, want[1])


def test_invalid_input_reported(ctx):
    xyz = np.zeros((10, 3), np.float32)
    xyz[3, 1] = np.nan
    f = N.Frame(ctx, N.default_params(0.01)).upload(xyz)
    with pytest.raises(N.PiError) as e:
        f.run()
    assert "PI_ERR_INVALID" in str(e.value)
    with pytest.raises(N.PiError) as e:
        N.Frame(ctx, N.default_params(0.01)).octree()
    assert "PI_ERR_STATE" in str(e.value)
