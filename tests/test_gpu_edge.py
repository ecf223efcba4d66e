"""Degenerate inputs on the GPU against the oracle: a single particle, ten
coincident particles (zero extent: the depth search starts at 0), particles on
a line and on a one-layer sheet (flat axes: one hash cell across, D_min =
D_max - 1; the line's last particle lies on the grid's upper bound, gets key
-1 and has no candidate within 4r, so its G is the identity), and a
non-finite coordinate (PI_ERR_INVALID)."""
import numpy as np
import pytest

import parity as PR
import pyoracle as O
from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B

pytestmark = pytest.mark.gpu

def _two_balls(gap):
    """Two jittered lattice balls (radius 0.1, spacing 0.02) `gap` apart: a
    root box of about gap / r leaf cells per axis, hence a deep octree."""
    rng = np.random.default_rng(5)
    g = np.arange(-0.1, 0.1001, 0.02)
    p = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    p = p[(p ** 2).sum(1) <= 0.1 ** 2]
    p = p + rng.uniform(-0.004, 0.004, p.shape)
    return np.concatenate([p, p + np.array([gap, 0.3 * gap, 0.1])]).astype(np.float32)


CASES = {
    "one": lambda: np.zeros((1, 3), np.float32) + 0.3,
    "coincident": lambda: np.zeros((10, 3), np.float32) + 0.3,
    "line": lambda: np.stack([np.linspace(0, 0.2, 11), np.zeros(11), np.zeros(11)], -1).astype(np.float32),
    "sheet": lambda: np.stack(np.meshgrid(np.arange(12) * 0.02, np.arange(12) * 0.02, [0.1], indexing="ij"),
                              -1).reshape(-1, 3).astype(np.float32),
    # D_max 11: the dual-vertex lattice is stored by occupied blocks
    "far_d11": lambda: _two_balls(15.0),
}


@pytest.fixture(scope="module")
def ctx():
    B.build()
    O.build()
    c = N.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", list(CASES))
def test_degenerate_frame_matches_oracle(ctx, name):
    xyz = CASES[name]()
    r = 0.01
    o = O.OracleFrame(xyz, r).run()
    g = N.Frame(ctx, N.default_params(r)).upload(xyz).run()
    info = g.info()
    d = o.depths()
    assert (info["depth_max"], info["depth_min"]) == (d["depth_max"], d["depth_min"])
    if name.startswith("far_d"):
        assert info["depth_max"] == int(name[len("far_d"):]), info["depth_max"]
    rep = PR.compare_octrees(o.nodes(), g.dump(N.DUMP_NODES), o, o.scalars()["max_scalar"], d["depth_min"])
    print(name, {k: v for k, v in rep.items() if k not in ("leaf_far_pos", "leaf_far_gpu", "unexplained")},
          rep["unexplained"][:4])
    assert not rep["unexplained"] and rep["nodes_oracle"] == rep["nodes_gpu"]
    vo, to, ko = o.mesh()
    vg, tg, kg = g.mesh(keys=True)
    mo = PR.canonical_mesh(vo, to, ko, one_based=True)
    mg = PR.canonical_mesh(vg, tg, kg, one_based=False)
    assert set(mo[0]) == set(mg[0]) and mo[1] == mg[1]
    g.close()


def test_depth_15_frame_close_to_oracle(ctx):
    """D_max 15: past D_max 14 the dual vertices come from sorted corner keys.
    The balls sit some 10^4 r from the origin, where a float coordinate
    resolves only about 1e-3 r, so the library (compensated sums, hi/lo
    centres) and the float oracle may disagree on samples near the
    isovalue: the octree sizes and meshes must agree to a small fraction,
    not node for node."""
    xyz = _two_balls(250.0)
    r = 0.01
    o = O.OracleFrame(xyz, r).run()
    g = N.Frame(ctx, N.default_params(r)).upload(xyz).run()
    info = g.info()
    assert info["depth_max"] == o.depths()["depth_max"] == 15
    n_o, n_g = len(o.nodes()["id"]), info["num_nodes"]
    assert abs(n_o - n_g) <= max(16, n_o // 50), (n_o, n_g)
    rep = PR.compare_meshes(o.mesh(), g.mesh(keys=True), r)
    print(rep)
    n_v = rep["verts_oracle"]
    assert n_v > 1000
    assert rep["verts_only_oracle"] + rep["verts_only_gpu"] <= n_v // 20
    assert rep["tris_only_oracle"] + rep["tris_only_gpu"] <= rep["tris_oracle"] // 20
    g.close()


def test_non_finite_coordinate_rejected(ctx):
    xyz = np.zeros((100, 3), np.float32)
    xyz[:, 0] = np.arange(100) * 0.02
    xyz[17, 1] = np.nan
    f = N.Frame(ctx, N.default_params(0.01)).upload(xyz)
    with pytest.raises(N.PiError) as e:
        f.run()
    assert e.value.code == N.PI_ERR_INVALID
    f.close()
    # the context still works afterwards
    xyz[17, 1] = 0.0
    f = N.Frame(ctx, N.default_params(0.01)).upload(xyz).run()
    assert f.info()["num_nodes"] > 0
    f.close()


def test_tiny_radius_rejected_before_keys(ctx):
    """A radius so small that a hash-grid axis would hold more cells than an
    int counts (the reference's int(ceil(...)) would overflow) is a size
    limit, reported before any key is computed; the context stays usable."""
    xyz = np.zeros((100, 3), np.float32)
    xyz[:, 0] = np.arange(100) * 0.02
    f = N.Frame(ctx, N.default_params(1e-20)).upload(xyz)
    with pytest.raises(N.PiError) as e:
        f.hashgrid()
    assert e.value.code == N.PI_ERR_LIMIT
    f.close()
    f = N.Frame(ctx, N.default_params(0.01)).upload(xyz).run()
    assert f.info()["num_nodes"] > 0
    f.close()


def test_zero_particles_rejected(ctx):
    f = N.Frame(ctx, N.default_params(0.01))
    with pytest.raises(N.PiError) as e:
        f.upload(np.zeros((0, 3), np.float32))
    assert e.value.code == N.PI_ERR_INVALID
    f.close()


def test_budget_exhausted_then_recovers():
    """A context whose byte budget is too small reports PI_ERR_NOMEM from the
    stage that overruns it, holds no bytes once the frame is gone, and the
    same input runs under a sufficient budget."""
    from particleisosurface_gb300 import synth
    fr = synth.small_blob(n=3000, seed=5)
    small = N.Context(0, budget_bytes=256 << 10)
    f = N.Frame(small, N.default_params(fr.radius)).upload(fr.xyz)
    with pytest.raises(N.PiError) as e:
        f.run()
    assert e.value.code == N.PI_ERR_NOMEM
    f.close()
    assert small.stats()["bytes"] == 0
    small.close()
    big = N.Context(0, budget_bytes=1 << 30)
    f = N.Frame(big, N.default_params(fr.radius)).upload(fr.xyz).run()
    assert f.info()["num_vertices"] > 0
    f.close()
    big.close()


def test_metrics_record_per_frame(tmp_path):
    """PISURF_METRICS names a file that receives one JSON line per frame."""
    import json
    import os
    import subprocess
    import sys
    out = tmp_path / "metrics.jsonl"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from particleisosurface_gb300 import _native as N, synth\n"
            "fr = synth.small_blob(n=2000, seed=3)\n"
            "c = N.Context(0)\n"
            "f = N.Frame(c, N.default_params(fr.radius)).upload(fr.xyz).run()\n"
            "f.reset().run()\n"
            "print(f.info()['num_triangles'])\n" % root)
    r = subprocess.run([sys.executable, "-c", code], env=dict(os.environ, PISURF_METRICS=str(out)),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(l) for l in out.read_text().splitlines()]
    assert len(lines) == 2
    assert lines[0]["triangles"] == int(r.stdout.strip().splitlines()[-1]) == lines[1]["triangles"]
    assert lines[0]["particles"] == 2000 and lines[0]["stage_ms"]["octree"] > 0


@pytest.mark.parametrize("name", ["one", "coincident", "line", "sheet"])
def test_degenerate_frame_qef_parts(ctx, name):
    """With the QEF on, a leaf level of a few nodes split into 64 parts (most
    of them empty) gives the nodes, QEF vertices and mesh of the level in one
    piece."""
    xyz = CASES[name]()
    p = N.default_params(0.01, qef=True)
    out = []
    for parts in (1, 64):
        ctx.tune_qef_parts(parts)
        g = N.Frame(ctx, p).upload(xyz).run()
        out.append((g.dump(N.DUMP_NODES).tobytes(), g.mesh(keys=True), g.info()["qef_accepted"]))
        g.close()
    ctx.tune_qef_parts(16)
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)
    assert out[0][2] == out[1][2]
