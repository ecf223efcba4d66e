"""GPU parity of splash particles (pi_params.splash) against the oracle with
PIO_SPLASH: the reference's GlobalSplash with its marking switched on
(src/evaluator.cpp:675,690) and GEN_SPLASH (src/surface_reconstructor.cpp:
299-320, Mesh::AppendSplash_ConstR, src/global.cpp:65-115).

  bit-exact: the splash flags and count; identity G, det 1 and zero normal
  of every splash particle; the appended icosahedra (positions, vertex
  keys, triangles);
  within the tolerances of tests/parity.py: G, determinants, normals and
  field values of the other particles (the field also against the GPU FP64
  oracle in splash mode); the octree node set and types; the surface mesh.
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
    "spray6k": lambda: synth.spray_frame(n=6000, seed=21),
    "blob2k": lambda: synth.small_blob(n=2000, seed=3),
    "spray20k": lambda: synth.spray_frame(n=20000, seed=23, radius=0.01),
}


@pytest.fixture(scope="module")
def ctx():
    B.build()
    O.build()
    c = N.Context(0)
    yield c
    c.close()


_cache = {}


def run_pair(ctx, name, qef=False):
    key = (name, qef)
    if key not in _cache:
        fr = CASES[name]()
        o = O.OracleFrame(fr.xyz, fr.radius, flags=O.SPLASH | (O.QEF if qef else 0)).run()
        o.frame_counts = (o.counter(0), o.counter(3))
        g = N.Frame(ctx, N.default_params(fr.radius, splash=True, qef=qef)).upload(fr.xyz).run()
        _cache[key] = (fr, o, g)
    return _cache[key]


@pytest.mark.parametrize("name", list(CASES))
def test_splash_flags_state_exact(ctx, name):
    fr, o, g = run_pair(ctx, name)
    sp = o.splash()
    gs = g.dump(N.DUMP_SPLASH)
    np.testing.assert_array_equal(gs, sp)
    ns = int(sp.sum())
    assert g.info()["num_splash"] == ns > 0
    m = sp.astype(bool)
    gG, gd, gn = g.dump(N.DUMP_G), g.dump(N.DUMP_DET), g.dump(N.DUMP_NORMALS)
    assert np.all(gG[m] == np.eye(3, dtype=np.float32)) and np.all(gd[m] == 1.0)
    assert np.all(gn[m] == 0.0)
    # the other particles as in the constant-radius parity tests
    o64 = O.OracleFrame(fr.xyz, fr.radius, flags=O.FP64 | O.SPLASH)
    for s in (1, 2, 3):
        o64.stage(s)
    np.testing.assert_array_equal(o64.splash(), sp)
    xm, G, det = o.aniso()
    x64, G64, d64 = o64.aniso()
    assert np.abs(gG[~m] - G64[~m]).max() <= PR.G_TOL
    assert np.all(np.abs(gG[~m] - G[~m]) <= np.abs(G[~m] - G64[~m]) + PR.G_TOL)
    n64 = o64.normals()
    scale = np.abs(n64).max()
    assert np.abs(gn - n64).max() <= PR.NORMAL_TOL * scale


@pytest.mark.parametrize("name", list(CASES))
def test_splash_field_skips_splash_particles(ctx, name):
    """Field values within tolerance of the oracle's (which skips splash
    particles, src/evaluator.cpp:73-76) and of the GPU FP64 oracle in
    splash mode; at a splash particle's own position its kernel is absent,
    so the field there is the sum of the other particles only."""
    fr, o, g = run_pair(ctx, name)
    sp = o.splash().astype(bool)
    rng = np.random.default_rng(3)
    pts = np.concatenate([fr.xyz[sp],
                          (fr.xyz[rng.choice(fr.n, 2000)] + rng.normal(0, 1.5 * fr.radius, (2000, 3))).astype(
                              np.float32)])
    ms = o.scalars()["max_scalar"]
    sg, so = g.eval(pts).astype(np.float64), o.eval(pts)
    s64 = g.eval_fp64(pts)
    o64 = O.OracleFrame(fr.xyz, fr.radius, flags=O.FP64 | O.SPLASH)
    for s in (1, 2, 3):
        o64.stage(s)
    np.testing.assert_allclose(s64, o64.eval(pts), rtol=0, atol=1e-10 * ms)
    e = np.abs(sg - s64) / ms
    print(name, "splash: field vs FP64 max %.3e, float reference %.3e" % (e.max(), (np.abs(so - s64) / ms).max()))
    assert e.max() <= PR.FIELD_TOL_FP64
    assert np.all(np.abs(sg - so) <= np.maximum(PR.FIELD_TOL * ms, np.abs(so - s64) + PR.FIELD_TOL_FP64 * ms))
    # an isolated splash particle (no other particle near) sees the iso value
    iso = g.info()["iso_value"]
    alone = sg[:int(sp.sum())][np.abs(so[:int(sp.sum())] - iso) == 0]
    assert np.all(alone == np.float32(iso))


def _check_icosahedra(o, g):
    """The last 12 ns vertices and 20 ns triangles, bit for bit."""
    ns = int(o.splash().sum())
    ov, ot, ok = o.mesh()
    gv, gt, gk = g.mesh(keys=True)
    info = g.info()
    assert info["num_vertices"] == len(gv) and info["num_triangles"] == len(gt)
    np.testing.assert_array_equal(gv[len(gv) - 12 * ns:], ov[len(ov) - 12 * ns:])
    np.testing.assert_array_equal(gk[len(gk) - 12 * ns:], ok[len(ok) - 12 * ns:])
    nvs_o, nvs_g = len(ov) - 12 * ns, len(gv) - 12 * ns
    np.testing.assert_array_equal(gt[len(gt) - 20 * ns:] - nvs_g, ot[len(ot) - 20 * ns:] - 1 - nvs_o)
    assert gt[:len(gt) - 20 * ns].max() < nvs_g


@pytest.mark.parametrize("name", list(CASES))
def test_splash_octree_and_mesh(ctx, name):
    fr, o, g = run_pair(ctx, name)
    ms = o.scalars()["max_scalar"]
    o64 = O.OracleFrame(fr.xyz, fr.radius, flags=O.FP64 | O.SPLASH)
    for s in (1, 2, 3):
        o64.stage(s)
    rep = PR.compare_octrees_fast(o.nodes(), g.dump(N.DUMP_NODES), o, ms, o.depths()["depth_min"],
                                  fp64_eval=o64.eval)
    print(name, {k: v for k, v in rep.items() if k != "unexplained"}, rep["unexplained"][:5])
    assert not rep["unexplained"]
    assert rep["explained"] <= max(2, rep["compared"] // 10000)
    _check_icosahedra(o, g)
    # the surface as in the constant-radius tests
    m = PR.compare_meshes_fast(o.mesh(), g.mesh(keys=True), fr.radius)
    print(name, {k: v for k, v in m.items() if k != "off_gpu_idx"})
    n_v = m["verts_oracle"]
    assert m["verts_only_oracle"] + m["verts_only_gpu"] <= max(4, n_v // 2000)
    assert m["tris_only_oracle"] + m["tris_only_gpu"] <= max(8, m["tris_oracle"] // 1000)
    agree, expl, bad = PR.check_vertices_fp64(g, m, fr.radius, ms, N.DUMP_NODES, N.DUMP_VERTEX_EDGES)
    assert len(bad) == 0, bad[:10]
    assert expl <= max(4, n_v // 2000)


def test_splash_with_qef(ctx):
    """Splash particles and the QEF together: the node set and types are the
    oracle's (the QEF moves leaf vertices, not the tree), the icosahedra are
    bit-exact and the surface mesh stays close (moved leaves change values
    near the surface, as in the QEF tests)."""
    fr, o, g = run_pair(ctx, "spray6k", qef=True)
    on = PR.node_table(o.nodes())
    gn = PR.node_table(g.dump(N.DUMP_NODES))
    assert set(on) == set(gn)
    assert all(on[k][0] == gn[k][0] for k in on)
    _check_icosahedra(o, g)
    m = PR.compare_meshes_fast(o.mesh(), g.mesh(keys=True), fr.radius)
    print(m)
    assert m["verts_only_oracle"] + m["verts_only_gpu"] <= max(8, m["verts_oracle"] // 50)


def test_splash_through_reconstruct_and_server(ctx):
    """pi_reconstruct (host in / host out, the triangle copy overlapping the
    bisection) and the request loop give the frame's mesh, icosahedra
    included."""
    fr, o, g = run_pair(ctx, "spray6k")
    gv, gt = g.mesh()
    p = N.default_params(fr.radius, splash=True)
    v, t = ctx.reconstruct(fr.xyz, p)
    np.testing.assert_array_equal(v, gv)
    np.testing.assert_array_equal(t, gt)
    srv = N.Server(0, slots=2)
    tk = srv.submit(fr.xyz, p)
    sv, st, _, _ = srv.result(tk)
    srv.close()
    np.testing.assert_array_equal(sv, gv)
    np.testing.assert_array_equal(st, gt)


def test_splash_off_changes_nothing(ctx):
    """With the flag off no particle is marked and the frame is the plain
    constant-radius frame; with it on, a frame without isolated particles
    gives the same surface."""
    fr = synth.spray_frame(n=4000, seed=24)
    g0 = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
    assert g0.info()["num_splash"] == 0 and not g0.dump(N.DUMP_SPLASH).any()
    ball = synth.slab_and_sphere(n=6000, seed=7)
    a = N.Frame(ctx, N.default_params(ball.radius)).upload(ball.xyz).run()
    b = N.Frame(ctx, N.default_params(ball.radius, splash=True)).upload(ball.xyz).run()
    if b.info()["num_splash"] == 0:
        for x, y in zip(a.mesh(keys=True), b.mesh(keys=True)):
            np.testing.assert_array_equal(x, y)
    for f in (g0, a, b):
        f.close()


def test_splash_rejected_with_per_particle_radii(ctx):
    fr = synth.small_blob(n=500, seed=13)
    f = N.Frame(ctx, N.default_params(fr.radius, splash=True)).upload(fr.xyz)
    with pytest.raises(N.PiError) as e:
        f.upload_radii(np.full(fr.n, fr.radius, np.float32))
    assert e.value.code == N.PI_ERR_INVALID
    f.close()
