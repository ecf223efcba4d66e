"""One field value per point, whatever the kernel: the octree's leaf values
come from the leaf-level and coarse-level thread-per-point kernels and from
the warp-per-chunk evaluation of the dense levels, pi_eval_field from its own
thread-per-point kernel.  All of them add the same in-support terms in
candidate order with the same compensated step, so a leaf's stored value
(SingleEval at its position) equals pi_eval_field there bit for bit."""
import numpy as np
import pytest

from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B
from particleisosurface_gb300 import synth

pytestmark = pytest.mark.gpu

T_LEAF = 2


@pytest.fixture(scope="module")
def ctx():
    B.build()
    c = N.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("qef", [False, True])
@pytest.mark.parametrize("case", ["slab_sphere_20k", "sheets_20k"])
def test_leaf_values_equal_point_evaluation(ctx, case, qef):
    fr = (synth.slab_and_sphere(n=20000, seed=1) if case == "slab_sphere_20k"
          else synth.sheets_and_filaments(n=20000, seed=9))
    g = N.Frame(ctx, N.default_params(fr.radius, qef=qef)).upload(fr.xyz).run()
    nodes = g.dump(N.DUMP_NODES)
    leaves = nodes[nodes["type"] == T_LEAF]
    if qef:
        # a QEF vertex moves the leaf's point; keep the leaves whose point is
        # still the centre (their value is SingleEval at the centre)
        leaves = leaves[np.all(leaves["node"][:, :3] == leaves["center"], axis=1)]
    assert len(leaves) > 1000
    depths = np.unique(leaves["depth"])
    assert len(depths) >= 2, depths  # leaves by size and by curvature
    pts = np.ascontiguousarray(leaves["node"][:, :3])
    val = g.eval(pts)
    stored = leaves["node"][:, 3]
    bad = np.nonzero(val.view(np.uint32) != stored.view(np.uint32))[0]
    assert len(bad) == 0, (len(bad), pts[bad[:3]], val[bad[:3]], stored[bad[:3]])
    g.close()


def test_leaf_values_equal_point_evaluation_at_full_size(ctx):
    """The same check on the 1M-particle dam-break frame (the benchmark's
    workload), on 200,000 leaves drawn at random: a size-independent
    property, where the oracle would take minutes."""
    fr = synth.dam_break(n=1_000_000, seed=2)
    g = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
    nodes = g.dump(N.DUMP_NODES)
    leaves = nodes[nodes["type"] == T_LEAF]
    assert len(leaves) > 1_000_000
    pick = np.random.default_rng(3).choice(len(leaves), 200_000, replace=False)
    leaves = leaves[pick]
    pts = np.ascontiguousarray(leaves["node"][:, :3])
    val = g.eval(pts)
    stored = leaves["node"][:, 3]
    assert np.array_equal(val.view(np.uint32), stored.view(np.uint32))
    g.close()


def test_octree_and_mesh_invariants_at_full_size(ctx):
    """Structural properties of the 1M frame's octree and mesh: levels are
    contiguous, every INTERNAL node has its 8 children (ids parent * 8 + k,
    centres parent +- half / 2) and no leaf has any; every mesh vertex lies
    on the segment between the positions of the two leaves of its key, and
    every triangle indexes existing vertices."""
    fr = synth.dam_break(n=1_000_000, seed=2)
    g = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
    nodes = g.dump(N.DUMP_NODES)
    v, t, k = g.mesh(keys=True)
    g.close()
    depth = nodes["depth"].astype(np.int64)
    assert np.all(np.diff(depth) >= 0)
    internal = np.nonzero(nodes["type"] == 1)[0]
    fc = nodes["first_child"]
    assert np.all(fc[nodes["type"] != 1] == -1)
    assert len(nodes) == 1 + 8 * len(internal)
    kids = fc[internal][:, None] + np.arange(8)[None, :]
    assert np.all(nodes["parent"][kids] == internal[:, None])
    assert np.all(nodes["id"][kids] == nodes["id"][internal][:, None] * 8 + np.arange(8, dtype=np.uint64))
    half = nodes["half"][internal][:, None, None]
    sign = np.array([[(1 if (q >> a) & 1 else -1) for a in range(3)] for q in range(8)], np.float32)
    want = nodes["center"][internal][:, None, :] + sign[None] * (half / 2)
    assert np.array_equal(nodes["center"][kids], want.astype(np.float32))
    # mesh: vertex on the segment between its two leaves' points (ids can
    # repeat across depths, as in the reference; vertices whose leaf ids
    # are not unique among the leaves are left out)
    leaf = np.nonzero(fc == -1)[0]
    order = leaf[np.argsort(nodes["id"][leaf], kind="stable")]
    ids = nodes["id"][order]
    uniq = np.ones(len(ids), bool)
    dup = ids[1:] == ids[:-1]
    uniq[1:] &= ~dup
    uniq[:-1] &= ~dup
    ia, ib = np.searchsorted(ids, k[:, 0]), np.searchsorted(ids, k[:, 1])
    assert np.all(ids[ia] == k[:, 0]) and np.all(ids[ib] == k[:, 1])
    keep = uniq[ia] & uniq[ib]
    assert keep.mean() > 0.99
    v = v[keep].astype(np.float64)
    a = nodes["node"][order[ia[keep]], :3].astype(np.float64)
    b = nodes["node"][order[ib[keep]], :3].astype(np.float64)
    ab = b - a
    s = np.einsum("ij,ij->i", v - a, ab) / np.einsum("ij,ij->i", ab, ab)
    off = np.linalg.norm(v - (a + s[:, None] * ab), axis=1)
    assert np.all((s > -1e-5) & (s < 1 + 1e-5)) and off.max() < 1e-3 * fr.radius, (s.min(), s.max(), off.max())
    # triangles index existing vertices (a triangle may repeat a vertex, as
    # the reference's do, where leaves of different sizes meet)
    assert t.min() >= 0 and t.max() < len(k)


@pytest.mark.parametrize("n", [20_000, 1_000_000])
def test_lattice_samples_equal_point_evaluation(ctx, n):
    """With the QEF on, every node sampled at depth >= D_min keeps its 27
    GridEval samples; on the two finest levels they come from the chunked
    evaluator (packed FP32 over pairs of candidates), elsewhere from the
    thread-per-point kernel.  Each equals pi_eval_field (the scalar field sum)
    at the same lattice point bit for bit."""
    import parity as PR
    fr = synth.slab_and_sphere(n=n, seed=1) if n <= 20_000 else synth.dam_break(n=n, seed=2)
    g = N.Frame(ctx, N.default_params(fr.radius, qef=True)).upload(fr.xyz).run()
    nodes = g.dump(N.DUMP_NODES)
    samp = g.dump(N.DUMP_QEF_SAMPLES).reshape(-1, 27)
    info = g.info()
    sampled = np.nonzero((nodes["depth"] >= info["depth_min"]) & (nodes["type"] != 0))[0]
    rng = np.random.default_rng(4)
    pick = rng.choice(sampled, size=min(len(sampled), 40_000), replace=False)
    # the finest two levels must be represented (chunked evaluation)
    assert set(np.unique(nodes["depth"][pick])) >= {info["depth_max"], info["depth_max"] - 1}
    pts = np.concatenate([PR.sample_points(nodes["center"][i], nodes["half"][i]) for i in pick])
    val = g.eval(pts).reshape(-1, 27)
    bad = np.nonzero(np.any(val.view(np.uint32) != samp[pick].view(np.uint32), axis=1))[0]
    assert len(bad) == 0, (len(bad), nodes["depth"][pick[bad[:5]]])
    g.close()


def bisect_f32(p, q, rr, eval32):
    """The library's edge bisection (calc_vertices, src/visitorextract.cpp:
    41-93) replayed on the host in float32 with every midpoint value from
    pi_eval_field: float midpoints, |p - q| as sqrt(x^2 + (y^2 + z^2)) halved
    per step, stop at length <= rr (at most 64 steps), ratio -p.w / (q.w -
    p.w), snapped to p below 0.1 and to q above 0.9 (compared in double, as
    the reference compares), else p + (q - p) * ratio.  p, q: (n, 4) float32
    node points (xyz, value)."""
    import parity as PR
    p = np.array(p, np.float32)
    q = np.array(q, np.float32)
    d = PR._fnorm(p[:, 0] - q[:, 0], p[:, 1] - q[:, 1], p[:, 2] - q[:, 2])
    rr = np.float32(rr)
    for _ in range(64):
        act = np.flatnonzero(d > rr)
        if len(act) == 0:
            break
        m = np.empty((len(act), 4), np.float32)
        m[:, :3] = (p[act, :3] + q[act, :3]) * np.float32(0.5)
        m[:, 3] = eval32(np.ascontiguousarray(m[:, :3]))
        keep_p = (m[:, 3] > 0) == (p[act, 3] > 0)
        p[act[keep_p]] = m[keep_p]
        q[act[~keep_p]] = m[~keep_p]
        d[act] = d[act] * np.float32(0.5)
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = (np.float32(0) - p[:, 3]) / (q[:, 3] - p[:, 3])
    v = p[:, :3] + (q[:, :3] - p[:, :3]) * ratio[:, None]
    lo, hi = ratio.astype(np.float64) < 0.1, ratio.astype(np.float64) > 0.9
    v[lo] = p[lo, :3]
    v[hi] = q[hi, :3]
    return v


@pytest.mark.parametrize("case", ["slab_sphere_20k", "sheets_20k", "spray_splash_20k", "dam_break_1m"])
def test_vertices_are_the_bisection_of_their_edges(ctx, case):
    """Every surface vertex is the float bisection of its edge (the two leaf
    points of PI_DUMP_VERTEX_EDGES) with each midpoint's value SingleEval at
    the midpoint, i.e. pi_eval_field there, bit for bit.  At 1M particles a
    size-independent property of the full frame."""
    splash = case == "spray_splash_20k"
    fr = {"slab_sphere_20k": lambda: synth.slab_and_sphere(n=20000, seed=1),
          "sheets_20k": lambda: synth.sheets_and_filaments(n=20000, seed=9),
          "spray_splash_20k": lambda: synth.spray_frame(n=20000, seed=23, radius=0.01),
          "dam_break_1m": lambda: synth.dam_break(n=1_000_000, seed=2)}[case]()
    g = N.Frame(ctx, N.default_params(fr.radius, splash=splash)).upload(fr.xyz).run()
    nodes = g.dump(N.DUMP_NODES)["node"]
    e = g.dump(N.DUMP_VERTEX_EDGES)
    v = g.mesh()[0]
    assert len(e) == len(v)
    # splash icosahedra (appended after the surface) have no edge
    ns = g.info()["num_splash"]
    assert (ns > 0) == splash and np.all(e[len(e) - 12 * ns:] == -1)
    e = e[:len(e) - 12 * ns]
    assert len(e) > 1000 and np.all(e >= 0)
    want = bisect_f32(nodes[e[:, 0]], nodes[e[:, 1]], np.float32(fr.radius) / np.float32(2), g.eval)
    got = v[:len(e)]
    bad = np.nonzero(np.any(got.view(np.uint32) != want.view(np.uint32), axis=1))[0]
    assert len(bad) == 0, (len(bad), len(e), got[bad[:3]], want[bad[:3]])
    g.close()


@pytest.mark.parametrize("case", ["slab_sphere_20k", "dam_break_1m"])
@pytest.mark.parametrize("qef", [False, True])
def test_run_and_staged_calls_give_the_same_mesh(ctx, case, qef):
    """pi_run starts the extraction's topology (leaf list, unique corners) on
    its own stream beside the octree's last level when the QEF is off; the
    staged calls (pi_octree_build, then pi_extract_mesh) run it inside the
    extraction.  Nodes and mesh are the same bit for bit either way."""
    fr = (synth.slab_and_sphere(n=20000, seed=1) if case == "slab_sphere_20k"
          else synth.dam_break(n=1_000_000, seed=2))
    p = N.default_params(fr.radius, qef=qef)
    a = N.Frame(ctx, p).upload(fr.xyz).run()
    b = N.Frame(ctx, p).upload(fr.xyz).hashgrid().aniso().normals()
    b.octree()
    b.extract()
    assert a.dump(N.DUMP_NODES).tobytes() == b.dump(N.DUMP_NODES).tobytes()
    for x, y in zip(a.mesh(keys=True), b.mesh(keys=True)):
        assert np.array_equal(x, y)
    assert a.info()["num_leaves"] == b.info()["num_leaves"] > 0
    a.close()
    b.close()
