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
    # a budget below two frames' estimates admits one frame at a time
    srv = N.Server(0, slots=4, budget_bytes=100 << 20)
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
