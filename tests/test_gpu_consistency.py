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
