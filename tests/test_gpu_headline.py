"""GPU parity at the headline configurations, against the oracle run on the
same seeded inputs (the comparison rules of test_gpu_parity.py, vectorised):

  dam_break_1m     1,000,000 particles, dam-break column + spray, r = 0.01
                   (the benchmark's frame), QEF off and on
  stress_500k      500,000 particles on thin sheets and filaments, r = 0.01
                   (near-degenerate covariances, ill-conditioned QEFs), QEF
                   off and on
  batch_frame      one frame of the 64-frame batched workload (about 300k
                   particles, a union of spheres and slabs)
  serving_frame    one request of the serving stream: step 25 of an advected
                   sequence, 158k particles, r = 0.005

Per case: hash keys, IndexList, cell offsets and neighbour lists bit-exact;
scalars and octree root exact; smoothed centres, G, determinants and normals
within tolerance of the float oracle; field, G and determinants against the
FP64 GPU oracle (max and RMS printed); octree node set and types identical
except near-isovalue / near-0.99-curvature nodes (counted, bounded); mesh
vertex keys, triangles and positions as in the small-frame tests.  With the
QEF on: accepted vertices within QEF_VERT_TOL * r of an FP64 solve of the
same samples, and the count of leaves the pseudo-inverse accepts where the
reference's float inverse rejects (the reference's accepted leaves must be
a subset).  Mirrors src/surface_reconstructor.cpp:409-479.
"""
import os

import numpy as np
import pytest

import parity as PR
import pyoracle as O
from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B
from particleisosurface_gb300 import synth

pytestmark = pytest.mark.gpu


def _serving_frame():
    reqs = synth.serving_requests(count=2000)
    req = next(r for r in reqs if r["seq"] == 12 and r["step"] == 25)
    return synth.serving_frame(req)


CASES = {
    "dam_break_1m": lambda: synth.dam_break(n=1_000_000, seed=2),
    "stress_500k": lambda: synth.sheets_and_filaments(n=500_000, seed=4),
    "batch_frame": lambda: synth.batch_frame(19),
    "serving_frame": _serving_frame,
}
RUNS = [("dam_break_1m", False), ("dam_break_1m", True), ("stress_500k", False), ("stress_500k", True),
        ("batch_frame", False), ("serving_frame", False)]
IDS = ["%s-qef%d" % (c, q) for c, q in RUNS]


@pytest.fixture(scope="module")
def ctx():
    B.build()
    O.build()
    O.set_threads(os.cpu_count() or 1)
    c = N.Context(0)
    yield c
    c.close()


_frames, _runs = {}, {}  # inputs by case; the live run (closed by its test)


def frame_of(name):
    if name not in _frames:
        _frames[name] = CASES[name]()
    return _frames[name]


def run(ctx, name, qef):
    """(frame, oracle, library frame) for one configuration, built once."""
    key = (name, qef)
    if key not in _runs:
        fr = frame_of(name)
        g = N.Frame(ctx, N.default_params(fr.radius, qef=qef)).upload(fr.xyz).run()
        o = O.OracleFrame(fr.xyz, fr.radius, flags=O.QEF if qef else 0).run()
        # the oracle's evaluation counters of the frame itself, before the
        # checks' own oracle evaluations add to them
        o.frame_counts = (o.counter(0), o.counter(3))
        _runs[key] = (fr, o, g)
    return _runs[key]


def _check_stages(fr, o, g):
    info = g.info()
    gi = o.grid_info()
    np.testing.assert_array_equal(np.array(info["bounding"], np.float32), gi["bounding"])
    assert info["cell_num"] == gi["cell_num"]
    np.testing.assert_array_equal(g.dump(N.DUMP_KEYS), o.keys())
    np.testing.assert_array_equal(g.dump(N.DUMP_INDEX_LIST), o.index_list())
    off = g.dump(N.DUMP_CELL_OFFSETS)
    h, s, e = o.cells()
    np.testing.assert_array_equal(off[h], s)
    np.testing.assert_array_equal(off[h + 1], e)
    rng = np.random.default_rng(11)
    pts = fr.xyz[rng.choice(fr.n, 300)]
    off_o, idx_o = o.neighbors(pts)
    off_g, idx_g = g.neighbors(pts)
    np.testing.assert_array_equal(off_g, off_o)
    np.testing.assert_array_equal(idx_g, idx_o)
    sc = o.scalars()
    d = o.depths()
    assert info["iso_value"] == np.float32(sc["iso"]) and info["max_scalar"] == np.float32(sc["max_scalar"])
    assert info["depth_max"] == d["depth_max"] and info["depth_min"] == d["depth_min"]
    np.testing.assert_array_equal(np.array(info["root_center"], np.float32), d["root_center"])
    assert info["root_half"] == np.float32(d["root_half"])


def _check_aniso_field(name, fr, o, g):
    # anisotropy against the float oracle (reference semantics) and the FP64
    # GPU oracle.  The float reference's own centres are a few float ulps off
    # FP64 (coordinates up to ~3.5 here, so ~1e-6 absolute, the size of
    # XMEAN_TOL * r); against it the bound is its own error plus ours.
    xm, G, det = o.aniso()
    gx, gG, gd = g.dump(N.DUMP_XMEANS), g.dump(N.DUMP_G).reshape(fr.n, 9), g.dump(N.DUMP_DET)
    x64, G64, d64 = g.aniso_fp64()
    Go = G.reshape(len(G), -1)
    assert np.all(np.abs(gx - xm) <= np.abs(xm - x64) + PR.XMEAN_TOL * fr.radius)
    assert np.all(np.abs(gG - Go) <= np.abs(Go - G64.reshape(len(G64), -1)) + PR.G_TOL)
    assert np.all(np.abs(gd - det) <= np.abs(det - d64) + PR.G_TOL)
    # normals (SingleEvalWithGrad at the particles) against the float oracle
    # and the FP64 oracle's gradient there, relative to the largest normal
    no = o.normals()
    gn = g.dump(N.DUMP_NORMALS)
    _, n64 = g.eval_fp64(fr.xyz, grad=True)
    scale = np.abs(n64).max()
    en = np.abs(gn - n64).max() / scale
    eno = np.abs(no - n64).max() / scale
    print("%s: normals vs FP64 max %.3e (float reference %.3e) of the largest" % (name, en, eno))
    assert en <= PR.NORMAL_TOL
    assert np.all(np.abs(gn - no) <= np.abs(no - n64) + PR.NORMAL_TOL * scale)
    eG = np.abs(gG - G64.reshape(len(G64), -1)).max(1)
    exo = np.abs(xm - x64).max(1) / fr.radius
    eGo = np.abs(G.reshape(len(G), -1) - G64.reshape(len(G64), -1)).max(1)
    ed = np.abs(gd - d64)
    ex = np.abs(gx - x64).max(1) / fr.radius
    flags = g.dump(N.DUMP_FP64_FLAGS).astype(bool)
    print("%s: G vs FP64 max %.3e rms %.3e (FP32 eigen path max %.3e, FP64 path max %.3e, %d of %d particles); "
          "float reference G vs FP64 max %.3e; det max %.3e; centres max %.3e r (float reference %.3e r)"
          % (name, eG.max(), np.sqrt(np.mean(eG ** 2)), eG[~flags].max() if (~flags).any() else 0.0,
             eG[flags].max() if flags.any() else 0.0, int(flags.sum()), fr.n, eGo.max(), ed.max(), ex.max(),
             exo.max()))
    assert eG.max() <= PR.G_TOL and ed.max() <= PR.G_TOL and ex.max() <= PR.XMEAN_TOL
    # field at points near the particles
    rng = np.random.default_rng(12)
    pts = (fr.xyz[rng.choice(fr.n, 20000)] + rng.normal(0, 1.5 * fr.radius, (20000, 3))).astype(np.float32)
    sg = g.eval(pts).astype(np.float64)
    s64 = g.eval_fp64(pts)
    so = o.eval(pts)
    ms = g.scalars_fp64()["max_scalar"]
    e = np.abs(sg - s64) / ms
    eo = np.abs(so - s64) / ms
    print("%s: field vs FP64 max %.3e rms %.3e (x MaxScalar); float reference max %.3e rms %.3e"
          % (name, e.max(), np.sqrt(np.mean(e ** 2)), eo.max(), np.sqrt(np.mean(eo ** 2))))
    assert e.max() <= PR.FIELD_TOL_FP64
    assert np.all(np.abs(sg - so) <= np.maximum(PR.FIELD_TOL * ms, np.abs(so - s64) + PR.FIELD_TOL_FP64 * ms))


def _check_octree_and_mesh(name, qef, fr, o, g):
    ms = o.scalars()["max_scalar"]
    on = o.nodes()
    gn = g.dump(N.DUMP_NODES)
    rep = PR.compare_octrees_fast(on, gn, o, ms, o.depths()["depth_min"], fp64_eval=g.eval_fp64)
    print(name, "qef" if qef else "", {k: v for k, v in rep.items() if k != "unexplained"}, rep["unexplained"][:5])
    assert not rep["unexplained"]
    assert rep["explained"] <= max(2, rep["compared"] // 10000)
    if not qef:
        # leaf values (at cell centres) beyond the float tolerance must sit
        # within the FP64 tolerance of the FP64 oracle
        assert rep["leaf_far_vs_fp64_max"] <= PR.FIELD_TOL_FP64
    # reference-equivalent evaluations of the octree: the SingleEval calls
    # the oracle makes (counter 0 minus its bisection calls, counter 3)
    info = g.info()
    ref_octree = o.frame_counts[0] - o.frame_counts[1]
    gpu_octree = info["field_evals"] - info["bisection_evals"]
    print(name, "qef" if qef else "", "octree evaluations: reference %d, library (reference-equivalent) %d, "
          "performed %d" % (ref_octree, gpu_octree, info["field_evals_performed"] - info["bisection_evals"]))
    if not qef and rep["explained"] == 0:
        assert gpu_octree == ref_octree
    m = PR.compare_meshes_fast(o.mesh(), g.mesh(keys=True), fr.radius)
    print(name, "qef" if qef else "", {k: v for k, v in m.items() if k != "off_gpu_idx"})
    n_v = m["verts_oracle"]
    assert n_v > 0
    if not qef:
        assert m["verts_only_oracle"] + m["verts_only_gpu"] <= max(4, n_v // 2000)
        assert m["tris_only_oracle"] + m["tris_only_gpu"] <= max(8, m["tris_oracle"] // 1000)
        # vertices off the float oracle's: the FP64 bisection of the same edge decides
        agree, expl, bad = PR.check_vertices_fp64(g, m, fr.radius, ms, N.DUMP_NODES, N.DUMP_VERTEX_EDGES)
        print(name, "vertices off the float oracle by > %g r: %d, of which %d agree with the FP64 bisection, "
              "%d at a near tie" % (PR.VERT_TOL, m["verts_off_tol"], agree, expl))
        assert len(bad) == 0, bad[:10]
        assert expl <= max(4, n_v // 2000)
    else:
        # moved leaves change values near the surface; the mesh stays close
        assert m["verts_only_oracle"] + m["verts_only_gpu"] <= max(8, n_v // 50)


def _check_qef_vertices(name, fr, o, g):
    gn = g.dump(N.DUMP_NODES)
    samp = g.dump(N.DUMP_QEF_SAMPLES).reshape(-1, 27)
    leaves = np.nonzero(gn["type"] == 2)[0]
    moved = np.any(gn["node"][:, :3] != gn["center"], axis=1)
    acc_g = leaves[moved[leaves]]
    info = g.info()
    assert len(acc_g) == info["qef_accepted"]
    # FP64 solve of the same samples: every accepted leaf plus a sample of the others
    rng = np.random.default_rng(13)
    rest = leaves[~moved[leaves]]
    pick = np.concatenate([acc_g, rng.choice(rest, size=min(100000, len(rest)), replace=False)])
    x, in_cell, singular = PR.qef_solve_f64_batch(gn["center"][pick], gn["half"][pick], samp[pick])
    acc64 = in_cell & ~singular
    mv = moved[pick]
    disagree = int(np.sum(acc64 != mv))
    both = acc64 & mv
    err = np.abs(gn["node"][pick[both]][:, :3] - x[both, :3]).max(1) / fr.radius
    # the reference's float inverse (the oracle with NodeCalcNode on): its
    # accepted leaves must be accepted here too; the count of leaves accepted
    # here and rejected there is the pseudo-inverse's departure
    on = o.nodes()
    ko = PR.node_keys(on["depth"], on["id"])
    kg = PR.node_keys(gn["depth"], gn["id"])
    _, io, ig = np.intersect1d(ko, kg, assume_unique=True, return_indices=True)
    lv = (on["type"][io] == 2) & (gn["type"][ig] == 2)
    mo = np.any(on["node"][io[lv], :3] != on["center"][io[lv]], axis=1)
    mg = moved[ig[lv]]
    only_here = int(np.sum(mg & ~mo))
    # leaves the reference's float inverse accepts and the library rejects:
    # the FP64 solve of the same samples must reject them too (a float
    # inverse of a matrix of condition ~1e20 can land inside the cell by
    # accident)
    ref_only = ig[lv][mo & ~mg]
    only_ref = len(ref_only)
    if only_ref:
        _, ic, sg = PR.qef_solve_f64_batch(gn["center"][ref_only], gn["half"][ref_only], samp[ref_only])
        assert not np.any(ic & ~sg), "leaves accepted by the reference and by the FP64 solve but not here"
    print("%s QEF: accepted %d (singular %d) of %d leaves; vs FP64 solve of %d leaves: max %.3e rms %.3e (x r), "
          "decision differs %d; float reference accepts %d, accepted here and rejected by the reference %d, "
          "accepted by the reference only %d (all rejected by the FP64 solve)"
          % (name, len(acc_g), info["qef_singular"], len(leaves), len(pick), err.max() if len(err) else 0.0,
             np.sqrt(np.mean(err ** 2)) if len(err) else 0.0, disagree, int(mo.sum()), only_here, only_ref))
    assert len(err) > 20 and err.max() <= PR.QEF_VERT_TOL
    assert disagree <= max(2, len(pick) // 1000)
    assert only_here == int(mg.sum()) - int(np.sum(mg & mo))


@pytest.mark.parametrize("name,qef", RUNS, ids=IDS)
def test_headline(ctx, name, qef):
    """Every check of one configuration on one library frame and one oracle
    run (a 1M-particle oracle frame takes a minute or two on the host cores)."""
    fr, o, g = run(ctx, name, qef)
    try:
        _check_stages(fr, o, g)
        if not qef:
            _check_aniso_field(name, fr, o, g)
        _check_octree_and_mesh(name, qef, fr, o, g)
        if qef:
            _check_qef_vertices(name, fr, o, g)
    finally:
        _runs.pop((name, qef))
        g.close()
        o.close()
