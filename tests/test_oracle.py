"""CPU tests of the oracle: known answers derived from the reference's math,
hand-placed hash keys (including its quirks), and the dual-marching-cubes
tables pinned to digests of the reference's own tables."""
import hashlib
import json
import os
import re

import numpy as np
import pytest

import pyoracle as O
from particleisosurface_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module", autouse=True)
def _build():
    O.build()


def _table_text(trans, flip, code):
    return "".join("%s,%d,%d;" % (",".join(map(str, trans[i])), int(flip[i]), int(code[i])) for i in range(256))


def test_dmc_table_matches_reference_digest():
    gold = json.load(open(os.path.join(HERE, "golden", "dmc_table.json")))
    t, f, c = O.dmc_table()
    assert hashlib.sha256(_table_text(t, f, c).encode()).hexdigest() == gold["table_sha256"]


def test_dmc_case_triangles_match_reference_digest():
    gold = json.load(open(os.path.join(HERE, "golden", "dmc_table.json")))
    h = open(os.path.join(HERE, "..", "oracle", "dmc_cases.h")).read()
    cases = {int(c, 16): [int(ch, 16) for ch in s] for c, s in re.findall(r'\{0x([0-9a-f]{2}), "([0-9a-f]+)"\}', h)}
    text = "".join("%d:%s;" % (code, ",".join(map(str, es))) for code, es in sorted(cases.items()))
    assert len(cases) == gold["num_cases"]
    assert hashlib.sha256(text.encode()).hexdigest() == gold["cases_sha256"]


def test_dmc_table_is_a_canonicalisation():
    """Every entry maps its code onto the canonical code by the permutation;
    flip is the orientation of the symmetry; 22 classes."""
    t, f, c = O.dmc_table()
    for idx in range(256):
        img = sum(((idx >> t[idx][i]) & 1) << i for i in range(8))
        assert img == c[idx]
        assert sorted(t[idx]) == list(range(8))
    assert len(set(c.tolist())) == 22


def _frame(xyz, r, flags=0):
    o = O.OracleFrame(np.asarray(xyz, np.float32), r, flags=flags)
    return o


def test_bspline_constants():
    """MaxScalar = Sigma (B(0) + 6 B(1) + 12 B(sqrt2) + 8 B(sqrt3)); iso = Sigma B(0.01);
    Influnce2 = (2r)^2; Sigma = (2r)^-6 (src/evaluator.cpp:5-58, 272-335)."""
    r = 0.025
    o = _frame([[0, 0, 0], [1, 1, 1], [0.5, 0.2, 0.7]], r)
    for s in (1, 2, 3):
        o.stage(s)
    sc = o.scalars()
    h = 2 * r
    assert sc["influence2"] == pytest.approx(h * h, rel=1e-6)
    assert sc["sigma"] == pytest.approx(h ** -6, rel=1e-6)

    def B(q):
        return 1 - 1.5 * q * q + 0.75 * q ** 3 if q <= 1 else (0.25 * (2 - q) ** 3 if q < 2 else 0.0)

    assert B(0) == 1 and B(2) == 0
    ms = sc["sigma"] * (B(0) + 6 * B(1) + 12 * B(2 ** 0.5) + 8 * B(3 ** 0.5))
    assert sc["max_scalar"] == pytest.approx(ms, rel=1e-6)
    assert sc["iso"] == pytest.approx(sc["sigma"] * B(0.01), rel=1e-6)


def test_isolated_particles_identity_g():
    r = 0.02
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.3, 0.7, 0.9]], np.float32)
    o = _frame(xyz, r)
    for s in (1, 2):
        o.stage(s)
    xm, g, det = o.aniso()
    np.testing.assert_allclose(xm, xyz, atol=0)
    for k in range(len(xyz)):
        np.testing.assert_allclose(g[k], np.eye(3), atol=1e-6)
    np.testing.assert_allclose(det, 1.0, atol=1e-6)


def test_interior_lattice_particle():
    """Perfect 2r lattice: an interior particle keeps x = p, G = I, and the
    field there is iso - MaxScalar.  (10 points per axis: with 9 the extent is
    a whole number of cells and the max-face particles get key -1.)"""
    r = 0.025
    k = np.arange(10) * 2 * r
    xyz = np.stack(np.meshgrid(k, k, k, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    o = _frame(xyz, r)
    for s in (1, 2, 3):
        o.stage(s)
    xm, g, det = o.aniso()
    c = 4 * 100 + 4 * 10 + 4  # particle (4, 4, 4)
    np.testing.assert_allclose(xm[c], xyz[c], atol=1e-6)
    np.testing.assert_allclose(g[c], np.eye(3), atol=1e-5)
    assert abs(det[c] - 1) < 1e-5
    sc = o.scalars()
    f = o.eval(xyz[c:c + 1])[0]
    assert f == pytest.approx(sc["iso"] - sc["max_scalar"], rel=1e-5)


def test_hash_keys_hand_placed():
    """Keys z*Nx*Ny + y*Nx + x of hand-placed points; int() truncates toward
    zero (src/hash_grid.cpp:124-139)."""
    r = 0.25  # cell 1.0
    xyz = np.array([[0.0, 0.0, 0.0], [2.5, 0.1, 0.2], [0.9, 1.9, 2.9], [3.0, 3.0, 3.0]], np.float32)
    o = _frame(xyz, r)
    o.stage(1)
    gi = o.grid_info()
    assert gi["cell_size"] == 1.0
    b = gi["bounding"]
    n = gi["xyz_cell_num"]
    # bbox [0,3]^3 has integral extent 3: Bounding = [0, 3], 3 cells per axis
    np.testing.assert_array_equal(b, [0, 3, 0, 3, 0, 3])
    np.testing.assert_array_equal(n, [3, 3, 3])
    keys = o.keys()
    exp = []
    for p in xyz:
        ix = [int((p[k] - b[2 * k]) / np.float32(1.0)) for k in range(3)]
        ok = all(0 <= ix[k] < n[k] for k in range(3))
        exp.append(ix[2] * 9 + ix[1] * 3 + ix[0] if ok else -1)
    np.testing.assert_array_equal(keys, exp)
    # the particle at the max corner falls on index 3 == XYZCellNum: key -1
    assert keys[3] == -1


def test_key_minus_one_shifts_cell_offsets():
    """With k particles of key -1, StartList/EndList count only valid keys but
    index IndexList, which holds the -1 particles first
    (src/hash_grid.cpp:103-162): cell lists are shifted by k."""
    r = 0.25
    xyz = np.array([[0.0, 0.0, 0.0], [1.5, 0.1, 0.1], [1.6, 0.2, 0.1], [3.0, 3.0, 3.0]], np.float32)
    o = _frame(xyz, r)
    o.stage(1)
    keys = o.keys()
    assert keys[3] == -1
    il = o.index_list()
    assert il[0] == 3  # key -1 sorts first
    h, s, e = o.cells()
    cells = dict(zip(h.tolist(), zip(s.tolist(), e.tolist())))
    assert cells[int(keys[0])] == (0, 1)
    assert cells[int(keys[1])] == (1, 3)
    # GetPIdxList around particle 0 returns IndexList[0:1] = particle 3 (shifted)
    off, nb = o.neighbors(xyz[:1])
    assert 3 in nb.tolist()


def test_oracle_runs_small_frame():
    fr = synth.small_blob(n=600, seed=11)
    o = O.OracleFrame(fr.xyz, fr.radius).run()
    v, t, k = o.mesh()
    assert len(v) > 0 and len(t) > 0
    assert t.min() >= 1 and t.max() <= len(v)
    d = o.depths()
    assert d["depth_min"] == d["depth_max"] - 3
    nd = o.nodes()
    # every INTERNAL node has 8 children, leaves none
    assert (nd["type"] == 1).sum() * 8 == len(nd["id"]) - 1


def test_stable_and_std_sort_agree_on_cells():
    fr = synth.small_blob(n=800, seed=5)
    a = O.OracleFrame(fr.xyz, fr.radius)
    b = O.OracleFrame(fr.xyz, fr.radius, flags=O.STD_SORT)
    a.stage(1)
    b.stage(1)
    np.testing.assert_array_equal(a.keys(), b.keys())
    ha, sa, ea = a.cells()
    hb, sb, eb = b.cells()
    np.testing.assert_array_equal(ha, hb)
    np.testing.assert_array_equal(sa, sb)
    il_a, il_b = a.index_list(), b.index_list()
    for s0, e0 in zip(sa, ea):
        assert sorted(il_a[s0:e0]) == sorted(il_b[s0:e0])


def test_uniform_grid_lattice_and_values():
    """UniformGrid (src/marching.cpp:42-93) in the oracle: the resized box,
    steps and dims follow the reference's float expressions, and each grid
    value is SingleEval at its lattice point."""
    fr = synth.small_blob(n=600, seed=21)
    o = O.OracleFrame(fr.xyz, fr.radius)
    for s in (1, 2, 3):
        o.stage(s)
    box, steps, dims = o.uniform_grid()
    f32 = np.float32
    xyz = fr.xyz
    r = f32(fr.radius)
    for a in range(3):
        mn, mx = xyz[:, a].min(), xyz[:, a].max()
        center = (mn + mx) / f32(2)
        length = mx - mn
        rl = f32(np.ceil(length / r)) * r + r * f32(4)
        assert box[2 * a] == center - rl / f32(2) and box[2 * a + 1] == center + rl / f32(2)
        assert steps[a] == int(rl / r) and dims[a] == steps[a] + 1
    vals = o.grid_sample()
    rng = np.random.default_rng(0)
    idx = [tuple(int(rng.integers(d)) for d in dims[::-1]) for _ in range(50)]

    def coord(a, i):
        st = f32(steps[a])
        return f32(f32(st - f32(i)) / st) * box[2 * a] + f32(f32(i) / st) * box[2 * a + 1]

    pts = np.array([[coord(0, x), coord(1, y), coord(2, z)] for z, y, x in idx], np.float32)
    ev = o.eval(pts)
    np.testing.assert_array_equal(np.array([vals[k] for k in idx]), ev)


def test_variable_radius_with_equal_radii_matches_constant_radius():
    """The variable-radius path (MultiLevelSearcher, per-particle kernel
    constants) with every radius equal: a single radius bin whose grid is the
    constant-radius grid, so keys, cell order, smoothed centres, G and the
    field are the constant-radius path's bit for bit (src/evaluator.cpp:16-37
    compute the same float constants either way)."""
    fr = synth.small_blob(n=1500, seed=5)
    c = O.OracleFrame(fr.xyz, fr.radius)
    v = O.OracleFrame(fr.xyz, np.full(fr.n, fr.radius, np.float32))
    for s in (1, 2):
        c.stage(s)
        v.stage(s)
    bins = v.bins()
    assert len(bins) == 1
    gi = c.grid_info()
    np.testing.assert_array_equal(bins[0]["bounding"], gi["bounding"])
    assert bins[0]["cell_num"] == gi["cell_num"]
    np.testing.assert_array_equal(bins[0]["keys"], c.keys())
    np.testing.assert_array_equal(bins[0]["index_list"], c.index_list())
    for a, b in zip(c.aniso(), v.aniso()):
        np.testing.assert_array_equal(a, b)
    rng = np.random.default_rng(1)
    pts = (fr.xyz[rng.choice(fr.n, 300)] + rng.normal(0, fr.radius, (300, 3))).astype(np.float32)
    off_c, idx_c = c.neighbors(pts)
    off_v, idx_v = v.neighbors(pts)
    np.testing.assert_array_equal(off_c, off_v)
    np.testing.assert_array_equal(idx_c, idx_v)
    # the searcher's radii: min * 0.99, max * 1.01
    sr = v.searcher_radii()
    assert sr["min"] == np.float32(np.float32(fr.radius) * 0.99) or abs(sr["min"] / fr.radius - 0.99) < 1e-6


def test_variable_radius_bins_and_frame():
    """Two radii, r and 2r: the searcher bins them (bin width about min / 2),
    each bin's grid has the cell size of its largest radius times 4, the
    neighbour list of a point is the bins' 27-cell lists in bin order, and a
    whole frame reconstructs (leaves at the depth of the smallest radius
    inside them)."""
    fr = synth.two_radius_frame(n=4000, seed=6)
    o = O.OracleFrame(fr.xyz, fr.radii)
    o.run()
    bins = o.bins()
    assert len(bins) == 2
    radii = fr.radii
    for b in bins:
        assert b["cell_size"] == np.float32(radii[b["radius_id"]] * np.float32(4.0))
        assert np.all(radii[b["particles"]] <= radii[b["radius_id"]])
        # IndexList is the bin's particles ordered by (key, particle)
        order = np.lexsort((b["particles"], b["keys"]))
        np.testing.assert_array_equal(b["index_list"], b["particles"][order])
    assert sum(len(b["particles"]) for b in bins) == fr.n
    v, t, k = o.mesh()
    assert len(v) > 100 and len(t) > 100
    nodes = o.nodes()
    leaves = nodes["type"] == 2
    assert leaves.any()


def test_splash_particles_marked_and_appended():
    """PIO_SPLASH: a particle is a splash particle exactly when it has <= 2
    candidates or <= 2 neighbours within 4r (src/evaluator.cpp:670-697 with
    the marking switched on); it keeps the identity G, has a zero normal,
    takes part in no field sum, and the mesh ends with one icosahedron of
    radius r per splash particle in particle order (12 vertices, 20
    triangles, src/global.cpp:94-115)."""
    fr = synth.spray_frame(n=3000, seed=22)
    xyz, r = fr.xyz, np.float32(fr.radius)
    o = O.OracleFrame(xyz, fr.radius, flags=O.SPLASH).run()
    sp = o.splash().astype(bool)
    # candidates and neighbours counted here, distances rounded as the
    # reference rounds them: x^2 + (y^2 + z^2) in float
    off, idx = o.neighbors(xyz)
    nI2 = np.float32(r * np.float32(4.0)) ** 2
    want = np.zeros(fr.n, bool)
    for i in range(fr.n):
        c = idx[off[i]:off[i + 1]]
        d = xyz[c] - xyz[i]
        d2 = d[:, 0] * d[:, 0] + (d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
        nn = int(np.count_nonzero((d2 < nI2) & (c != i)))
        want[i] = len(c) <= 2 or nn <= 2
    np.testing.assert_array_equal(sp, want)
    ns = int(sp.sum())
    assert 20 < ns < fr.n // 5
    xm, G, det = o.aniso()
    assert np.all(G[sp] == np.eye(3)) and np.all(det[sp] == 1.0)
    assert np.all(o.normals()[sp] == 0.0)
    v, t, k = o.mesh()
    vs, ts, ks = v[-12 * ns:], t[-20 * ns:], k[-12 * ns:]
    d = np.linalg.norm(vs.reshape(ns, 12, 3) - xyz[sp][:, None, :], axis=2)
    assert np.abs(d / r - 1.0).max() < 1e-5
    pid = np.flatnonzero(sp)
    np.testing.assert_array_equal(ks[:, 0], (12 * pid[:, None] + np.arange(12)).ravel())
    assert np.all(ks[:, 1] == np.iinfo(np.uint64).max)
    first = len(v) - 12 * ns + 1  # 1-based, as Mesh::tris
    tri0 = ts[:20] - first
    assert tri0.min() == 0 and tri0.max() == 11
    # a closed surface: every edge of an icosahedron is in two triangles
    edges = {}
    for a, b, c in tri0:
        for e in ((a, b), (b, c), (c, a)):
            edges[tuple(sorted(e))] = edges.get(tuple(sorted(e)), 0) + 1
    assert len(edges) == 30 and set(edges.values()) == {2}
    # without the flag nothing is marked and no key is a splash key
    o0 = O.OracleFrame(xyz, fr.radius).run()
    assert o0.splash().sum() == 0
    assert not np.any(o0.mesh()[2][:, 1] == np.iinfo(np.uint64).max)
