"""ctypes binding of the CPU oracle (test infrastructure only).

Only the tests, the smoke check and the benchmark's CPU-baseline leg import
this module; the shipped library never does.  `build()` compiles the oracle
with make into oracle/_build/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpioracle.so")

STD_SORT = 1
QEF = 2
FP64 = 4
SPLASH = 8

_lib = None


def build(quiet=True):
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        fp = C.POINTER(C.c_float)
        dp = C.POINTER(C.c_double)
        i64 = C.c_int64
        sig = {
            "pio_create": (P, [fp, i64, C.c_float, C.c_float, C.c_float, C.c_int]),
            "pio_destroy": (None, [P]),
            "pio_set_threads": (None, [C.c_int]),
            "pio_stage": (C.c_int, [P, C.c_int]),
            "pio_run": (C.c_int, [P]),
            "pio_stage_seconds": (C.c_double, [P, C.c_int]),
            "pio_counter": (i64, [P, C.c_int]),
            "pio_grid_info": (C.c_int, [P, fp, C.POINTER(i64), C.POINTER(i64), fp]),
            "pio_get_keys": (C.c_int, [P, C.POINTER(i64)]),
            "pio_get_index_list": (C.c_int, [P, C.POINTER(C.c_int32)]),
            "pio_num_cells": (i64, [P]),
            "pio_get_cells": (C.c_int, [P, C.POINTER(i64), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
            "pio_neighbors": (i64, [P, fp, i64, C.POINTER(i64), C.POINTER(C.c_int32), i64]),
            "pio_in_box": (i64, [P, fp, fp, C.POINTER(C.c_int32), i64]),
            "pio_get_aniso": (C.c_int, [P, dp, dp, dp]),
            "pio_get_normals": (C.c_int, [P, dp]),
            "pio_get_splash": (C.c_int, [P, C.POINTER(C.c_int8)]),
            "pio_scalars": (C.c_int, [P, dp]),
            "pio_depths": (C.c_int, [P, C.POINTER(C.c_int32), fp, fp]),
            "pio_eval": (C.c_int, [P, fp, i64, dp, dp]),
            "pio_num_nodes": (i64, [P]),
            "pio_get_nodes": (C.c_int, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_int8), C.POINTER(C.c_int8),
                                        fp, fp, fp, fp, C.POINTER(C.c_int8), C.POINTER(C.c_int32)]),
            "pio_mesh_counts": (C.c_int, [P, C.POINTER(i64), C.POINTER(i64)]),
            "pio_mesh_get": (C.c_int, [P, fp, C.POINTER(C.c_int32), C.POINTER(C.c_uint64)]),
            "pio_write_obj": (C.c_int, [P, C.c_char_p]),
            "pio_dmc_table": (C.c_int, [C.POINTER(C.c_int32), C.POINTER(C.c_int8), C.POINTER(C.c_int32)]),
            "pio_uniform_grid": (C.c_int, [P, fp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
            "pio_grid_sample": (C.c_int, [P, dp, i64]),
            "pio_create_var": (P, [fp, fp, i64, C.c_float, C.c_float, C.c_int]),
            "pio_num_bins": (C.c_int, [P]),
            "pio_bin_info": (C.c_int, [P, C.c_int, fp, C.POINTER(i64), C.POINTER(i64), fp, C.POINTER(i64),
                                       C.POINTER(C.c_int32)]),
            "pio_bin_lists": (C.c_int, [P, C.c_int, C.POINTER(C.c_int32), C.POINTER(i64), C.POINTER(C.c_int32)]),
            "pio_searcher_radii": (C.c_int, [P, fp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def dmc_table():
    t = np.zeros((256, 8), np.int32)
    f = np.zeros(256, np.int8)
    c = np.zeros(256, np.int32)
    lib().pio_dmc_table(_p(t, C.c_int32), _p(f, C.c_int8), _p(c, C.c_int32))
    return t, f.astype(bool), c


def set_threads(n):
    lib().pio_set_threads(int(n))


class OracleFrame:
    """One reconstruction (SurfReconstructor + Run) on the CPU oracle."""

    def __init__(self, xyz, radius, smooth_factor=2.0, iso_factor=1.9, flags=0):
        """radius: a float (constant radius) or an array of per-particle radii
        (the variable-radius path)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        self.n = xyz.shape[0]
        self.flags = flags
        if np.ndim(radius) == 0:
            self.h = lib().pio_create(_p(xyz, C.c_float), self.n, radius, smooth_factor, iso_factor, flags)
        else:
            r = np.ascontiguousarray(radius, dtype=np.float32)
            assert r.shape == (self.n,)
            self.h = lib().pio_create_var(_p(xyz, C.c_float), _p(r, C.c_float), self.n, smooth_factor, iso_factor,
                                          flags)

    def close(self):
        if self.h:
            lib().pio_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stage(self, s):
        rc = lib().pio_stage(self.h, s)
        if rc:
            raise RuntimeError("oracle stage %d failed: %d" % (s, rc))

    def run(self):
        rc = lib().pio_run(self.h)
        if rc:
            raise RuntimeError("oracle run failed: %d" % rc)
        return self

    def seconds(self, s):
        return lib().pio_stage_seconds(self.h, s)

    def counter(self, w):
        return lib().pio_counter(self.h, w)

    def grid_info(self):
        b = np.zeros(6, np.float32)
        x = np.zeros(3, np.int64)
        cn = C.c_int64()
        cs = C.c_float()
        lib().pio_grid_info(self.h, _p(b, C.c_float), _p(x, C.c_int64), C.byref(cn), C.byref(cs))
        return dict(bounding=b, xyz_cell_num=x, cell_num=cn.value, cell_size=cs.value)

    def bins(self):
        """Per grid (one for a constant radius, else one per non-empty radius
        bin): dict of bounding, xyz_cell_num, cell_num, cell_size, radius_id,
        particles (bin-local order), keys, index_list (particle indices)."""
        out = []
        for b in range(lib().pio_num_bins(self.h)):
            bb = np.zeros(6, np.float32)
            x = np.zeros(3, np.int64)
            cn, cnt = C.c_int64(), C.c_int64()
            cs = C.c_float()
            rid = C.c_int32()
            lib().pio_bin_info(self.h, b, _p(bb, C.c_float), _p(x, C.c_int64), C.byref(cn), C.byref(cs),
                               C.byref(cnt), C.byref(rid))
            parts = np.zeros(cnt.value, np.int32)
            keys = np.zeros(cnt.value, np.int64)
            il = np.zeros(cnt.value, np.int32)
            lib().pio_bin_lists(self.h, b, _p(parts, C.c_int32), _p(keys, C.c_int64), _p(il, C.c_int32))
            out.append(dict(bounding=bb, xyz_cell_num=x, cell_num=cn.value, cell_size=cs.value,
                            radius_id=rid.value, particles=parts, keys=keys, index_list=il))
        return out

    def searcher_radii(self):
        o = np.zeros(3, np.float32)
        rc = lib().pio_searcher_radii(self.h, _p(o, C.c_float))
        return None if rc else dict(min=o[0], max=o[1], avg=o[2])

    def keys(self):
        k = np.zeros(self.n, np.int64)
        lib().pio_get_keys(self.h, _p(k, C.c_int64))
        return k

    def index_list(self):
        k = np.zeros(self.n, np.int32)
        lib().pio_get_index_list(self.h, _p(k, C.c_int32))
        return k

    def cells(self):
        m = lib().pio_num_cells(self.h)
        h = np.zeros(m, np.int64)
        s = np.zeros(m, np.int32)
        e = np.zeros(m, np.int32)
        lib().pio_get_cells(self.h, _p(h, C.c_int64), _p(s, C.c_int32), _p(e, C.c_int32))
        return h, s, e

    def neighbors(self, pts):
        pts = np.ascontiguousarray(pts, dtype=np.float32)
        m = pts.shape[0]
        cap = max(1024, m * 512)
        while True:
            off = np.zeros(m + 1, np.int64)
            out = np.zeros(cap, np.int32)
            tot = lib().pio_neighbors(self.h, _p(pts, C.c_float), m, _p(off, C.c_int64), _p(out, C.c_int32), cap)
            if tot >= 0:
                return off, out[:tot]
            cap *= 4

    def in_box(self, b1, b2):
        b1 = np.ascontiguousarray(b1, dtype=np.float32)
        b2 = np.ascontiguousarray(b2, dtype=np.float32)
        cap = self.n * 2 + 16
        out = np.zeros(cap, np.int32)
        tot = lib().pio_in_box(self.h, _p(b1, C.c_float), _p(b2, C.c_float), _p(out, C.c_int32), cap)
        return out[:tot]

    def aniso(self):
        xm = np.zeros((self.n, 3))
        g = np.zeros((self.n, 3, 3))
        d = np.zeros(self.n)
        lib().pio_get_aniso(self.h, _p(xm, C.c_double), _p(g, C.c_double), _p(d, C.c_double))
        return xm, g, d

    def splash(self):
        out = np.zeros(self.n, np.int8)
        assert lib().pio_get_splash(self.h, _p(out, C.c_int8)) == 0
        return out

    def normals(self):
        nr = np.zeros((self.n, 3))
        lib().pio_get_normals(self.h, _p(nr, C.c_double))
        return nr

    def scalars(self):
        o = np.zeros(4)
        lib().pio_scalars(self.h, _p(o, C.c_double))
        return dict(iso=o[0], max_scalar=o[1], influence2=o[2], sigma=o[3])

    def depths(self):
        d = np.zeros(2, np.int32)
        c = np.zeros(3, np.float32)
        h = C.c_float()
        lib().pio_depths(self.h, _p(d, C.c_int32), _p(c, C.c_float), C.byref(h))
        return dict(depth_max=int(d[0]), depth_min=int(d[1]), root_center=c, root_half=h.value)

    def eval(self, pts, grad=False):
        pts = np.ascontiguousarray(pts, dtype=np.float32)
        m = pts.shape[0]
        s = np.zeros(m)
        g = np.zeros((m, 3)) if grad else None
        rc = lib().pio_eval(self.h, _p(pts, C.c_float), m, _p(s, C.c_double),
                            _p(g, C.c_double) if grad else None)
        if rc:
            raise RuntimeError("oracle eval before normals stage")
        return (s, g) if grad else s

    def uniform_grid(self):
        """UniformGrid's lattice: box (6), steps (3), dims (3)."""
        box = np.zeros(6, np.float32)
        steps = np.zeros(3, np.int32)
        dims = np.zeros(3, np.int32)
        rc = lib().pio_uniform_grid(self.h, _p(box, C.c_float), _p(steps, C.c_int32), _p(dims, C.c_int32))
        if rc:
            raise RuntimeError("oracle uniform grid before stage 1")
        return box, steps, dims

    def grid_sample(self):
        """UniformGrid::gridSampling: values[dims[2], dims[1], dims[0]] (float64)."""
        box, steps, dims = self.uniform_grid()
        out = np.zeros(int(dims[0]) * int(dims[1]) * int(dims[2]))
        rc = lib().pio_grid_sample(self.h, _p(out, C.c_double), out.size)
        if rc:
            raise RuntimeError("oracle grid sampling before stage 3")
        return out.reshape(int(dims[2]), int(dims[1]), int(dims[0]))

    def nodes(self):
        m = lib().pio_num_nodes(self.h)
        out = dict(
            id=np.zeros(m, np.uint64), depth=np.zeros(m, np.int8), type=np.zeros(m, np.int8),
            node=np.zeros((m, 4), np.float32), center=np.zeros((m, 3), np.float32),
            half=np.zeros(m, np.float32), curv=np.zeros(m, np.float32),
            signchange=np.zeros(m, np.int8), parent=np.zeros(m, np.int32))
        lib().pio_get_nodes(self.h, _p(out["id"], C.c_uint64), _p(out["depth"], C.c_int8),
                            _p(out["type"], C.c_int8), _p(out["node"], C.c_float),
                            _p(out["center"], C.c_float), _p(out["half"], C.c_float),
                            _p(out["curv"], C.c_float), _p(out["signchange"], C.c_int8),
                            _p(out["parent"], C.c_int32))
        return out

    def mesh(self):
        nv = C.c_int64()
        nt = C.c_int64()
        lib().pio_mesh_counts(self.h, C.byref(nv), C.byref(nt))
        v = np.zeros((nv.value, 3), np.float32)
        t = np.zeros((nt.value, 3), np.int32)
        k = np.zeros((nv.value, 2), np.uint64)
        lib().pio_mesh_get(self.h, _p(v, C.c_float), _p(t, C.c_int32), _p(k, C.c_uint64))
        return v, t, k

    def write_obj(self, path):
        return lib().pio_write_obj(self.h, path.encode())
