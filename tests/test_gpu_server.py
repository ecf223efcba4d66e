"""GPU test of the request loop (pi_server_*): frames submitted together run
concurrently on the device, and each frame's mesh is the same as when it is
reconstructed alone (pi_run on its own context) -- bit for bit, since a
frame's computation does not depend on what runs beside it."""
import numpy as np
import pytest

from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B
from particleisosurface_gb300 import synth

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix():
    B.build()
    frames = [synth.mixed_frame(700 + k, n) for k, n in enumerate([20000, 60000, 9000, 120000, 35000, 70000])]
    frames.append(synth.small_blob(n=3000, seed=41))
    ctx = N.Context(0)
    alone = []
    for fr in frames:
        f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
        alone.append(f.mesh())
        f.close()
    srv = N.Server(0, slots=4, budget_bytes=0)
    tickets = [srv.submit(fr.xyz, N.default_params(fr.radius)) for fr in frames]
    mixed = [srv.result(t) for t in tickets]
    st = srv.stats()
    srv.close()
    ctx.close()
    assert st["completed"] == len(frames)
    assert st["max_in_flight"] >= 2, st
    for (va, ta), (vm, tm, lat, q) in zip(alone, mixed):
        np.testing.assert_array_equal(vm, va)
        np.testing.assert_array_equal(tm, ta)
        assert lat >= q >= 0


def test_budget_admission_serialises_large_requests():
    B.build()
    frames = [synth.mixed_frame(800 + k, 40000) for k in range(4)]
    # a budget below two frames' reservations admits one frame at a time
    # (reservation 40000 * 3072 B + 128 MiB each)
    srv = N.Server(0, slots=4, budget_bytes=400 << 20)
    tickets = [srv.submit(fr.xyz, N.default_params(fr.radius)) for fr in frames]
    for t in tickets:
        srv.result(t)
    st = srv.stats()
    srv.close()
    assert st["completed"] == 4 and st["max_in_flight"] == 1, st


def test_failed_request_reports_its_error_and_others_complete():
    B.build()
    good = synth.small_blob(n=3000, seed=43)
    bad = N.default_params(good.radius)
    bad.max_depth = 2  # the frame needs a deeper octree: PI_ERR_LIMIT inside the worker
    srv = N.Server(0, slots=2, budget_bytes=0)
    t_bad = srv.submit(good.xyz, bad)
    t_good = srv.submit(good.xyz, N.default_params(good.radius))
    with pytest.raises(N.PiError) as ei:
        srv.result(t_bad)
    assert ei.value.code == N.PI_ERR_LIMIT
    v, t, lat, q = srv.result(t_good)
    srv.close()
    assert len(v) > 0 and len(t) > 0


def _alone(fr):
    ctx = N.Context(0)
    f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
    m = f.mesh()
    f.close()
    ctx.close()
    return m


def test_sequence_steps_reuse_their_resident_frame():
    """Steps of advected sequences submitted one after another: each step
    runs in the resident frame of its sequence's previous step and gives
    what a fresh frame gives."""
    B.build()
    base = [synth.mixed_frame(900 + k, n) for k, n in enumerate([15000, 40000])]
    steps = []
    for k, fr in enumerate(base):
        p = fr.xyz64
        for st in range(4):
            if st:
                p = synth.advect(p, 1.0, synth.SERVE_G, (st - 1) * synth.SERVE_DT, synth.SERVE_DT, scale=fr.scale)
            steps.append((k + 1, np.ascontiguousarray(p.astype(np.float32)), fr.radius))
    srv = N.Server(0, slots=4, budget_bytes=0)
    out = []
    for seq, xyz, r in steps:  # one at a time: the holder of the sequence is idle
        out.append(srv.result(srv.submit(xyz, N.default_params(r), seq=seq)))
    info = srv.info()
    srv.close()
    assert info["completed"] == len(steps)
    assert info["resident_hits"] == len(steps) - len(base), info
    for (seq, xyz, r), (v, t, lat, q) in zip(steps, out):
        fr = synth.Frame(xyz.astype(np.float64), r, 1.0, 0, "step")
        va, ta = _alone(fr)
        np.testing.assert_array_equal(v, va)
        np.testing.assert_array_equal(t, ta)


def test_small_requests_pass_a_blocked_head_within_the_bound():
    """With a budget that holds one large frame, small requests queued behind
    a large one that cannot start yet pass it; the large one is passed a
    bounded number of times and completes; every result equals the frame
    reconstructed alone."""
    B.build()
    big = [synth.mixed_frame(950 + k, 150000) for k in range(2)]
    small = [synth.small_blob(n=2000, seed=960 + k) for k in range(6)]
    est = lambda n: n * 3072 + (128 << 20)  # the default reservation
    srv = N.Server(0, slots=4, budget_bytes=int(est(150000) + 3 * est(2000)))
    frames = [big[0], big[1]] + small
    tickets = [srv.submit(fr.xyz, N.default_params(fr.radius)) for fr in frames]
    res = [srv.result(t) for t in tickets]
    info = srv.info()
    srv.close()
    assert info["completed"] == len(frames) and info["bypasses"] >= 1, info
    assert info["bypasses"] <= 8 * len(frames)
    for fr, (v, t, lat, q) in zip(frames, res):
        va, ta = _alone(fr)
        np.testing.assert_array_equal(v, va)
        np.testing.assert_array_equal(t, ta)


def test_underestimated_request_is_requeued_with_a_larger_reservation():
    """A reservation below what the frame needs: the frame's context is capped
    at it, the frame fails inside the worker, and the request goes back to the
    head of the queue with twice the reservation until it fits; the result is
    the frame's as reconstructed alone.  Beyond the whole budget the request
    fails with PI_ERR_NOMEM."""
    B.build()
    fr = synth.mixed_frame(970, 60000)
    srv = N.Server(0, slots=2, budget_bytes=1 << 30)
    srv.set_estimate(64, 1 << 20)  # far below the frame's needs
    v, t, lat, q = srv.result(srv.submit(fr.xyz, N.default_params(fr.radius)))
    info = srv.info()
    va, ta = _alone(fr)
    np.testing.assert_array_equal(v, va)
    np.testing.assert_array_equal(t, ta)
    assert info["retries"] >= 1, info
    srv.close()
    # a budget too small for the frame at all
    srv = N.Server(0, slots=2, budget_bytes=8 << 20)
    srv.set_estimate(64, 1 << 20)
    with pytest.raises(N.PiError) as e:
        srv.result(srv.submit(fr.xyz, N.default_params(fr.radius)))
    assert e.value.code == N.PI_ERR_NOMEM
    srv.close()
