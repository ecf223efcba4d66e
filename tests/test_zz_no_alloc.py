"""GPU test of pi_hashgrid_build_noalloc, the hash-grid build for callers that
cannot allow the library to allocate device memory (programs that hold the
whole GPU in their own pool, or that forbid allocation after start-up).

It calls the entry point through the C ABI twice in a row on different
frames, with device buffers the test owns, and checks each result against
the regular allocating build (pi_hashgrid_build and its dumps).  The results
are integers (cell keys, cell order, cell offsets), so the check is exact.
This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B
from particleisosurface_gb300 import synth

pytestmark = pytest.mark.gpu


def _noalloc_fn():
    fn = N.lib().pi_hashgrid_build_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int64, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                   C.POINTER(C.c_float), C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.c_void_p]
    return fn


def test_noalloc_hashgrid_matches_allocating_build_twice():
    torch = pytest.importorskip("torch")
    B.build()
    fn = _noalloc_fn()
    ctx = N.Context(0)
    frames = [synth.small_blob(n=4000, seed=31), synth.slab_and_sphere(n=9000, seed=32)]
    for k, fr in enumerate(frames):
        ref = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).hashgrid()
        keys_ref = ref.dump(N.DUMP_KEYS)
        il_ref = ref.dump(N.DUMP_INDEX_LIST)
        off_ref = ref.dump(N.DUMP_CELL_OFFSETS)
        info = ref.info()

        n = fr.n
        d_xyz = torch.from_numpy(fr.xyz.copy()).cuda()
        d_keys = torch.full((n,), 7, dtype=torch.int32, device="cuda")
        d_il = torch.full((n,), 7, dtype=torch.int32, device="cuda")
        d_off = torch.full((len(off_ref),), 7, dtype=torch.int32, device="cuda")
        bnd = (C.c_float * 6)()
        xyz_n = (C.c_int32 * 3)()
        cn = C.c_int64()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = fn(d_xyz.data_ptr(), n, fr.radius, d_keys.data_ptr(), d_il.data_ptr(), d_off.data_ptr(),
                len(off_ref), bnd, xyz_n, C.byref(cn), None)
        assert rc == 0, N.lib().pi_last_error()
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if k > 0:
            # the first call was the warm-up (it may load the library's device
            # code); every later call leaves the device's free memory as it was
            assert free_after == free_before, (free_before, free_after)
        np.testing.assert_array_equal(np.array(bnd[:], np.float32), np.array(info["bounding"], np.float32))
        assert list(xyz_n) == list(info["xyz_cell_num"]) and cn.value == info["cell_num"]
        np.testing.assert_array_equal(d_keys.cpu().numpy().astype(np.int64), keys_ref)
        np.testing.assert_array_equal(d_il.cpu().numpy(), il_ref)
        np.testing.assert_array_equal(d_off.cpu().numpy(), off_ref)
        ref.close()
    ctx.close()


def test_noalloc_rejects_sizes_beyond_limit():
    torch = pytest.importorskip("torch")
    B.build()
    fn = _noalloc_fn()
    fr = synth.small_blob(n=1000, seed=33)
    d_xyz = torch.from_numpy(fr.xyz.copy()).cuda()
    d_keys = torch.zeros(fr.n, dtype=torch.int32, device="cuda")
    d_il = torch.zeros(fr.n, dtype=torch.int32, device="cuda")
    d_off = torch.zeros(16, dtype=torch.int32, device="cuda")
    bnd = (C.c_float * 6)()
    xyz_n = (C.c_int32 * 3)()
    cn = C.c_int64()
    # too many particles: rejected on the host before any device work
    rc = fn(d_xyz.data_ptr(), 1048577, fr.radius, d_keys.data_ptr(), d_il.data_ptr(), d_off.data_ptr(), 16, bnd,
            xyz_n, C.byref(cn), None)
    assert rc == -5 and b"exceed" in N.lib().pi_last_error()
    # cell offset buffer too short: rejected with the needed count, before keys are written
    rc = fn(d_xyz.data_ptr(), fr.n, fr.radius, d_keys.data_ptr(), d_il.data_ptr(), d_off.data_ptr(), 16, bnd,
            xyz_n, C.byref(cn), None)
    assert rc == -5 and cn.value + 1 > 16
    # a radius so small that an axis of the hash grid would hold more cells
    # than an int can count: rejected before any key is computed
    rc = fn(d_xyz.data_ptr(), fr.n, 1e-20, d_keys.data_ptr(), d_il.data_ptr(), d_off.data_ptr(), 16, bnd,
            xyz_n, C.byref(cn), None)
    assert rc == -5 and b"exceeds the limit" in N.lib().pi_last_error() and cn.value == -1
    torch.cuda.synchronize()
