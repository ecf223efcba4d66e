"""Samples per lane of the chunked field evaluation (pi_ctx_tune): K = 1, 2
and 4 chunk the same distinct samples differently, and each sample's sum runs
over the same candidates in the same order, so every node value, the octree
and the mesh are bit-identical whatever K, with and without the QEF leaves.
The timed choice (K = 0) settles on one of 1, 2, 4 per level kind."""
import numpy as np
import pytest

from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B
from particleisosurface_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    B.build()
    c = N.Context(0)
    yield c
    c.close()


def run_frame(ctx, fr, qef, k):
    ctx.tune(k)
    g = N.Frame(ctx, N.default_params(fr.radius, qef=qef)).upload(fr.xyz).run()
    nodes = g.dump(N.DUMP_NODES)
    v, t = g.mesh()
    tuning = ctx.tuning()
    g.close()
    return nodes, v, t, tuning


@pytest.mark.parametrize("qef", [False, True])
def test_samples_per_lane_change_no_result(ctx, qef):
    fr = synth.slab_and_sphere(n=20000, seed=1)
    ref = run_frame(ctx, fr, qef, 1)
    assert ref[3] == [1, 1]
    for k in (2, 4, 0):
        nodes, v, t, tuning = run_frame(ctx, fr, qef, k)
        assert nodes.tobytes() == ref[0].tobytes(), k
        assert np.array_equal(v, ref[1]) and np.array_equal(t, ref[2]), k
        if k:
            assert tuning == [k, k]
        else:
            # without QEF the leaf level evaluates node centres only (no
            # chunked evaluation there), so only the level above is timed
            assert tuning[0] in ((1, 2, 4) if qef else (0,)) and tuning[1] in (1, 2, 4)
    ctx.tune(0)


@pytest.mark.parametrize("qef", [False, True])
def test_every_evaluation_configuration_gives_the_same_frame(ctx, qef):
    """Warps per block and staged candidates per warp (with K, the table the
    timing chooses from) change neither a node nor the mesh."""
    fr = synth.slab_and_sphere(n=20000, seed=1)
    ref = run_frame(ctx, fr, qef, 2)
    seen = set()
    nconf = N.Context.eval_configs()
    assert nconf >= 8
    for i in range(nconf):
        ctx.tune_config(i)
        g = N.Frame(ctx, N.default_params(fr.radius, qef=qef)).upload(fr.xyz).run()
        nodes = g.dump(N.DUMP_NODES)
        v, t = g.mesh()
        cfg = ctx.tuning_config()
        g.close()
        assert nodes.tobytes() == ref[0].tobytes(), i
        assert np.array_equal(v, ref[1]) and np.array_equal(t, ref[2]), i
        assert cfg[0] == cfg[1]
        seen.add(cfg[1])
    assert len(seen) == nconf and any(c[3] for c in seen)
    ctx.tune_config(-1)
    g = N.Frame(ctx, N.default_params(fr.radius, qef=qef)).upload(fr.xyz).run()
    assert g.dump(N.DUMP_NODES).tobytes() == ref[0].tobytes()
    assert ctx.tuning_config()[1] in seen
    g.close()
    ctx.tune(0)


def test_tune_rejects_other_values(ctx):
    for k in (3, 8, -1):
        with pytest.raises(N.PiError):
            ctx.tune(k)
    for i in (N.Context.eval_configs(), -2):
        with pytest.raises(N.PiError):
            ctx.tune_config(i)
    ctx.tune(0)


@pytest.mark.parametrize("case", ["slab20k", "blob2k"])
def test_qef_parts_change_no_result(ctx, case):
    """The leaf level with the QEF on in 1 to 64 parts (each part's QEF on the
    QEF stream beside the next part's sampling, pi_ctx_tune_qef_parts): nodes,
    QEF vertices, the QEF counts and the mesh are the same bit for bit; a
    small frame leaves most of 64 parts empty."""
    fr = synth.slab_and_sphere(n=20000, seed=1) if case == "slab20k" else synth.small_blob(n=2000, seed=3)
    assert ctx.qef_parts() == 16

    def run(parts):
        ctx.tune_qef_parts(parts)
        g = N.Frame(ctx, N.default_params(fr.radius, qef=True)).upload(fr.xyz).run()
        out = (g.dump(N.DUMP_NODES).tobytes(), g.mesh(), g.info())
        g.close()
        return out

    ref = run(1)
    assert ref[2]["qef_accepted"] > 0
    for parts in (2, 3, 16, 64):
        nodes, (v, t), info = run(parts)
        assert nodes == ref[0], parts
        assert np.array_equal(v, ref[1][0]) and np.array_equal(t, ref[1][1]), parts
        assert (info["qef_accepted"], info["qef_singular"]) == (ref[2]["qef_accepted"], ref[2]["qef_singular"])
    ctx.tune_qef_parts(16)


def test_qef_parts_rejects_other_values(ctx):
    for parts in (0, -1, 65):
        with pytest.raises(N.PiError) as e:
            ctx.tune_qef_parts(parts)
        assert e.value.code == N.PI_ERR_INVALID
    assert ctx.qef_parts() == 16
