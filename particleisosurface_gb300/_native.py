"""ctypes binding of libpisurf.so (the C ABI in include/pisurf.h).

The library is the only compute path: there is no CPU fallback.  Loading fails
with an ImportError naming the missing file if the extension has not been
built, and every computing call raises PiError if CUDA is unavailable.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libpisurf.so")

PI_OK = 0
PI_OK, PI_ERR_INVALID, PI_ERR_CUDA, PI_ERR_NOMEM, PI_ERR_STATE, PI_ERR_LIMIT = 0, -1, -2, -3, -4, -5
ERRORS = {-1: "PI_ERR_INVALID", -2: "PI_ERR_CUDA", -3: "PI_ERR_NOMEM", -4: "PI_ERR_STATE", -5: "PI_ERR_LIMIT"}

DUMP_KEYS, DUMP_INDEX_LIST, DUMP_CELL_OFFSETS, DUMP_XMEANS, DUMP_G, DUMP_DET, DUMP_NORMALS, DUMP_NODES, \
    DUMP_FP64_FLAGS, DUMP_QEF_SAMPLES, DUMP_GRID_OF, DUMP_SPLASH, DUMP_VERTEX_EDGES = range(1, 14)


class PiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, code), msg))
        self.code = code


class Params(C.Structure):
    _fields_ = [("radius", C.c_float), ("smooth_factor", C.c_float), ("iso_factor", C.c_float),
                ("qef", C.c_int32), ("max_depth", C.c_int32), ("splash", C.c_int32),
                ("reserved", C.c_int32 * 6)]


class FrameInfo(C.Structure):
    _fields_ = [("num_particles", C.c_int64), ("num_invalid_keys", C.c_int64), ("bounding", C.c_float * 6),
                ("cell_size", C.c_float), ("xyz_cell_num", C.c_int32 * 3), ("cell_num", C.c_int64),
                ("depth_max", C.c_int32), ("depth_min", C.c_int32), ("root_center", C.c_float * 3),
                ("root_half", C.c_float), ("iso_value", C.c_float), ("max_scalar", C.c_float),
                ("influence2", C.c_float), ("sigma", C.c_float), ("num_nodes", C.c_int64),
                ("num_leaves", C.c_int64), ("num_empty", C.c_int64), ("num_dual_cells", C.c_int64),
                ("num_vertices", C.c_int64), ("num_triangles", C.c_int64), ("field_evals", C.c_int64),
                ("candidate_pairs", C.c_int64), ("bisection_evals", C.c_int64), ("fp64_eigen", C.c_int64),
                ("stage_ms", C.c_float * 8), ("qef_accepted", C.c_int64), ("qef_singular", C.c_int64),
                ("grid_pairs", C.c_int64), ("field_evals_performed", C.c_int64), ("num_grids", C.c_int32),
                ("radius_min", C.c_float), ("radius_max", C.c_float), ("num_splash", C.c_int64)]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


NODE_DTYPE = np.dtype([("id", np.uint64), ("center", np.float32, 3), ("half", np.float32),
                       ("node", np.float32, 4), ("curv", np.float32), ("parent", np.int32),
                       ("first_child", np.int32), ("depth", np.int8), ("type", np.int8),
                       ("signchange", np.int8), ("pad", np.int8)])

_lib = None


def _declare(L):
    P = C.c_void_p
    PP = C.POINTER(C.c_void_p)
    fp = C.POINTER(C.c_float)
    i64 = C.c_int64
    pi64 = C.POINTER(C.c_int64)
    sig = {
        "pi_last_error": (C.c_char_p, []),
        "pi_version": (C.c_char_p, []),
        "pi_params_default": (None, [C.POINTER(Params)]),
        "pi_ctx_create": (C.c_int, [C.c_int, C.c_size_t, PP]),
        "pi_ctx_destroy": (C.c_int, [P]),
        "pi_ctx_stats": (C.c_int, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
        "pi_ctx_profile": (C.c_int, [P, C.c_int]),
        "pi_ctx_kernel_time": (C.c_int, [P, C.POINTER(C.c_double), pi64, pi64, pi64]),
        "pi_ctx_kernel_groups": (C.c_int, [P, C.c_int32, C.POINTER(C.c_double), pi64, pi64, pi64]),
        "pi_ctx_stream": (P, [P]),
        "pi_ctx_tune": (C.c_int, [P, C.c_int32]),
        "pi_ctx_tuning": (C.c_int, [P, C.POINTER(C.c_int32)]),
        "pi_ctx_tuning_config": (C.c_int, [P, C.POINTER(C.c_int32)]),
        "pi_ctx_tune_config": (C.c_int, [P, C.c_int32]),
        "pi_ctx_tune_qef_parts": (C.c_int, [P, C.c_int32]),
        "pi_ctx_qef_parts": (C.c_int, [P, C.POINTER(C.c_int32)]),
        "pi_eval_configs": (C.c_int, []),
        "pi_frame_create": (C.c_int, [P, C.POINTER(Params), PP]),
        "pi_frame_destroy": (C.c_int, [P]),
        "pi_frame_upload": (C.c_int, [P, fp, i64]),
        "pi_frame_upload_device": (C.c_int, [P, P, i64]),
        "pi_frame_reset": (C.c_int, [P]),
        "pi_frame_upload_radii": (C.c_int, [P, fp, i64]),
        "pi_frame_grid": (C.c_int, [P, C.c_int32, fp, C.POINTER(C.c_int32), fp, pi64, pi64, C.POINTER(C.c_int32)]),
        "pi_hashgrid_build": (C.c_int, [P]),
        "pi_aniso_compute": (C.c_int, [P]),
        "pi_normals_compute": (C.c_int, [P]),
        "pi_octree_build": (C.c_int, [P]),
        "pi_extract_mesh": (C.c_int, [P]),
        "pi_run": (C.c_int, [P]),
        "pi_frame_info_get": (C.c_int, [P, C.POINTER(FrameInfo)]),
        "pi_mesh_counts": (C.c_int, [P, pi64, pi64]),
        "pi_mesh_get": (C.c_int, [P, fp, C.POINTER(C.c_int32), C.POINTER(C.c_uint64)]),
        "pi_mesh_write_obj": (C.c_int, [P, C.c_char_p]),
        "pi_eval_field": (C.c_int, [P, fp, i64, fp, fp]),
        "pi_fp64_aniso": (C.c_int, [P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "pi_fp64_eval_field": (C.c_int, [P, fp, i64, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "pi_fp64_scalars": (C.c_int, [P, C.POINTER(C.c_double)]),
        "pi_grid_dims": (C.c_int, [P, C.POINTER(C.c_int32), fp, pi64]),
        "pi_load_csv": (C.c_int, [C.c_char_p, fp, fp, i64, pi64, C.POINTER(C.c_int32)]),
        "pi_load_hdf5": (C.c_int, [C.c_char_p, fp, fp, i64, pi64]),
        "pi_hdf5_dataset": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_double), i64, pi64, pi64,
                                      C.POINTER(C.c_int32)]),
        "pi_load_xdmf": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.c_char_p, i64, pi64,
                                   C.POINTER(C.c_int32)]),
        "pi_write_ply": (C.c_int, [C.c_char_p, fp, i64, C.POINTER(C.c_int32), i64, C.c_int32]),
        "pi_mesh_write_ply": (C.c_int, [P, C.c_char_p]),
        "pi_grid_sample": (C.c_int, [P, fp, i64]),
        "pi_grid_sample_device": (C.c_int, [P, C.c_void_p, i64]),
        "pi_grid_write_vti": (C.c_int, [P, C.c_char_p]),
        "pi_hashgrid_neighbors": (C.c_int, [P, fp, i64, pi64, C.POINTER(C.c_int32), i64, pi64]),
        "pi_hashgrid_in_box": (C.c_int, [P, fp, fp, C.POINTER(C.c_int32), i64, pi64]),
        "pi_stage_dump_size": (C.c_int, [P, C.c_int, C.POINTER(C.c_size_t)]),
        "pi_stage_dump": (C.c_int, [P, C.c_int, P, C.c_size_t]),
        "pi_reconstruct": (C.c_int, [P, C.POINTER(Params), fp, i64, fp, i64, C.POINTER(C.c_int32), i64, pi64,
                                     pi64]),
        "pi_dmc_table": (C.c_int, [C.POINTER(C.c_int32), C.POINTER(C.c_int8), C.POINTER(C.c_int32)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libpisurf.so is not built (%s); run particleisosurface_gb300/build.py" % LIB_PATH)
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def check(rc):
    if rc != PI_OK:
        raise PiError(rc, lib().pi_last_error().decode(errors="replace"))


def ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def default_params(radius, smooth_factor=2.0, iso_factor=1.9, qef=False, max_depth=0, splash=False):
    p = Params()
    lib().pi_params_default(C.byref(p))
    p.radius = radius
    p.smooth_factor = smooth_factor
    p.iso_factor = iso_factor
    p.qef = 1 if qef else 0
    p.max_depth = max_depth
    p.splash = 1 if splash else 0
    return p


def dmc_table():
    t = np.zeros((256, 8), np.int32)
    f = np.zeros(256, np.int8)
    c = np.zeros(256, np.int32)
    check(lib().pi_dmc_table(ptr(t, C.c_int32), ptr(f, C.c_int8), ptr(c, C.c_int32)))
    return t, f.astype(bool), c


def load_csv(path, radius=False):
    """loadParticlesFromCSV: (xyz float32 [n, 3], radius float32 [n] or None,
    column indices x, y, z, radius)."""
    n = C.c_int64()
    cols = np.zeros(4, np.int32)
    check(lib().pi_load_csv(str(path).encode(), None, None, 0, C.byref(n), ptr(cols, C.c_int32)))
    xyz = np.empty((n.value, 3), np.float32)
    rad = np.empty(n.value, np.float32) if radius else None
    check(lib().pi_load_csv(str(path).encode(), ptr(xyz, C.c_float), ptr(rad, C.c_float) if radius else None,
                            n.value, C.byref(n), ptr(cols, C.c_int32)))
    return xyz, rad, cols


def load_hdf5(path, radius=False):
    """readShonDyParticleData: (xyz float32 [n, 3], radius float32 [n] or None)."""
    n = C.c_int64()
    check(lib().pi_load_hdf5(str(path).encode(), None, None, 0, C.byref(n)))
    xyz = np.empty((n.value, 3), np.float32)
    rad = np.empty(n.value, np.float32) if radius else None
    check(lib().pi_load_hdf5(str(path).encode(), ptr(xyz, C.c_float), ptr(rad, C.c_float) if radius else None,
                             n.value, C.byref(n)))
    return xyz, rad


def hdf5_dataset(path, name):
    """One dataset of an HDF5 file as float64, shaped by its dataspace."""
    cnt = C.c_int64()
    dims = np.zeros(8, np.int64)
    rank = C.c_int32()
    check(lib().pi_hdf5_dataset(str(path).encode(), name.encode(), None, 0, C.byref(cnt), ptr(dims, C.c_int64),
                                C.byref(rank)))
    out = np.empty(cnt.value, np.float64)
    check(lib().pi_hdf5_dataset(str(path).encode(), name.encode(), ptr(out, C.c_double), cnt.value, C.byref(cnt),
                                None, None))
    return out.reshape(tuple(int(d) for d in dims[:rank.value]))


def load_xdmf(directory, xdmf_file, target_frame=0):
    """readShonDyParticleXDMF: the frame file names of an XDMF frame list."""
    ln = C.c_int64()
    nf = C.c_int32()
    check(lib().pi_load_xdmf(str(directory).encode(), str(xdmf_file).encode(), target_frame, None, 0, C.byref(ln),
                             C.byref(nf)))
    buf = C.create_string_buffer(ln.value)
    check(lib().pi_load_xdmf(str(directory).encode(), str(xdmf_file).encode(), target_frame, buf, ln.value,
                             C.byref(ln), C.byref(nf)))
    s = buf.value.decode()
    return s.split("\n") if nf.value else []


def write_ply(path, verts, tris, one_based=False):
    """writePlyFile: binary PLY (float32 vertices, uchar/int face lists)."""
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
    check(lib().pi_write_ply(str(path).encode(), ptr(v, C.c_float), v.shape[0], ptr(t, C.c_int32), t.shape[0],
                             1 if one_based else 0))


class Context:
    """One GPU, one stream (pi_ctx)."""

    def __init__(self, device=0, budget_bytes=0):
        h = C.c_void_p()
        check(lib().pi_ctx_create(device, budget_bytes, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().pi_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self):
        a = C.c_uint64()
        b = C.c_uint64()
        check(lib().pi_ctx_stats(self.h, C.byref(a), C.byref(b)))
        return dict(launches=a.value, bytes=b.value)

    def tune(self, samples_per_lane=0):
        """Fix the chunked evaluation's samples per lane (1, 2 or 4); 0 = time them."""
        check(lib().pi_ctx_tune(self.h, samples_per_lane))

    def tuning(self):
        """[leaf level, level above]: samples per lane in use, 0 = not chosen yet."""
        out = (C.c_int32 * 2)()
        check(lib().pi_ctx_tuning(self.h, out))
        return [out[0], out[1]]

    def tuning_config(self):
        """[leaf level, level above]: (K, warps per block, staged candidates, bulk staging) in use."""
        out = (C.c_int32 * 8)()
        check(lib().pi_ctx_tuning_config(self.h, out))
        return [tuple(out[0:4]), tuple(out[4:8])]

    @staticmethod
    def eval_configs():
        return lib().pi_eval_configs()

    def tune_config(self, index):
        """Fix entry `index` of the evaluation configuration table; -1 = time them."""
        check(lib().pi_ctx_tune_config(self.h, index))

    def tune_qef_parts(self, parts):
        """Parts of the leaf level pipelined against the QEF stream (QEF on);
        1 = one piece.  Changes no result."""
        check(lib().pi_ctx_tune_qef_parts(self.h, parts))

    def qef_parts(self):
        v = C.c_int32()
        check(lib().pi_ctx_qef_parts(self.h, C.byref(v)))
        return v.value

    def profile(self, enable=True):
        check(lib().pi_ctx_profile(self.h, 1 if enable else 0))

    def kernel_time(self):
        ms = C.c_double()
        n = C.c_int64()
        p = C.c_int64()
        e = C.c_int64()
        check(lib().pi_ctx_kernel_time(self.h, C.byref(ms), C.byref(n), C.byref(p), C.byref(e)))
        return dict(ms=ms.value, launches=n.value, pairs=p.value, evals=e.value)

    GROUPS = ("chunked_sampling", "per_sample_sampling", "leaf_values", "bisection", "qef", "uniform_grid")

    def kernel_groups(self):
        """Per kernel group (GROUPS order): dict of ms, launches, pairs, units
        accumulated since the last read (pi_ctx_kernel_groups)."""
        n = len(self.GROUPS)
        ms = (C.c_double * n)()
        la, pa, un = (C.c_int64 * n)(), (C.c_int64 * n)(), (C.c_int64 * n)()
        check(lib().pi_ctx_kernel_groups(self.h, n, ms, la, pa, un))
        return {g: dict(ms=ms[k], launches=la[k], pairs=pa[k], units=un[k]) for k, g in enumerate(self.GROUPS)}

    def reconstruct(self, xyz, params, max_verts=None, max_tris=None):
        """Host in / host out: pi_reconstruct."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        n = xyz.shape[0]
        mv = max_verts or max(1024, 4 * n)
        mt = max_tris or 2 * mv
        while True:
            v = np.empty((mv, 3), np.float32)
            t = np.empty((mt, 3), np.int32)
            nv = C.c_int64()
            nt = C.c_int64()
            rc = lib().pi_reconstruct(self.h, C.byref(params), ptr(xyz, C.c_float), n, ptr(v, C.c_float), mv,
                                      ptr(t, C.c_int32), mt, C.byref(nv), C.byref(nt))
            if rc == -5 and (nv.value > mv or nt.value > mt):
                mv, mt = max(mv, nv.value), max(mt, nt.value)
                continue
            check(rc)
            return v[:nv.value], t[:nt.value]


class Frame:
    """One reconstruction's device state (pi_frame)."""

    def __init__(self, ctx, params):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().pi_frame_create(ctx.h, C.byref(params), C.byref(h)))
        self.h = h
        self.n = 0

    def close(self):
        if self.h:
            lib().pi_frame_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        self.n = xyz.shape[0]
        check(lib().pi_frame_upload(self.h, ptr(xyz, C.c_float), self.n))
        return self

    def upload_radii(self, radii):
        """Per-particle radii (pi_frame_upload_radii): the variable-radius path."""
        r = np.ascontiguousarray(radii, dtype=np.float32)
        check(lib().pi_frame_upload_radii(self.h, ptr(r, C.c_float), r.shape[0]))
        return self

    def grid(self, k):
        """Hash grid k (pi_frame_grid): bounding, dims, cell_size, count,
        offset_base, radius_id."""
        b = np.zeros(6, np.float32)
        d = np.zeros(3, np.int32)
        cs = C.c_float()
        cnt, ob = C.c_int64(), C.c_int64()
        rid = C.c_int32()
        check(lib().pi_frame_grid(self.h, k, ptr(b, C.c_float), ptr(d, C.c_int32), C.byref(cs), C.byref(cnt),
                                  C.byref(ob), C.byref(rid)))
        return dict(bounding=b, dims=d, cell_size=cs.value, count=cnt.value, offset_base=ob.value,
                    radius_id=rid.value)

    def upload_device(self, dptr, n):
        self.n = n
        check(lib().pi_frame_upload_device(self.h, C.c_void_p(dptr), n))
        return self

    def reset(self):
        check(lib().pi_frame_reset(self.h))
        return self

    def hashgrid(self):
        check(lib().pi_hashgrid_build(self.h))
        return self

    def aniso(self):
        check(lib().pi_aniso_compute(self.h))
        return self

    def normals(self):
        check(lib().pi_normals_compute(self.h))
        return self

    def octree(self):
        check(lib().pi_octree_build(self.h))
        return self

    def extract(self):
        check(lib().pi_extract_mesh(self.h))
        return self

    def run(self):
        check(lib().pi_run(self.h))
        return self

    def info(self):
        fi = FrameInfo()
        check(lib().pi_frame_info_get(self.h, C.byref(fi)))
        return fi.as_dict()

    def mesh(self, keys=False):
        nv = C.c_int64()
        nt = C.c_int64()
        check(lib().pi_mesh_counts(self.h, C.byref(nv), C.byref(nt)))
        v = np.empty((nv.value, 3), np.float32)
        t = np.empty((nt.value, 3), np.int32)
        k = np.empty((nv.value, 2), np.uint64) if keys else None
        check(lib().pi_mesh_get(self.h, ptr(v, C.c_float), ptr(t, C.c_int32),
                                ptr(k, C.c_uint64) if keys else None))
        return (v, t, k) if keys else (v, t)

    def write_obj(self, path):
        check(lib().pi_mesh_write_obj(self.h, path.encode()))

    def eval(self, pts, grad=False):
        pts = np.ascontiguousarray(pts, dtype=np.float32)
        m = pts.shape[0]
        s = np.empty(m, np.float32)
        g = np.empty((m, 3), np.float32) if grad else None
        check(lib().pi_eval_field(self.h, ptr(pts, C.c_float), m, ptr(s, C.c_float),
                                  ptr(g, C.c_float) if grad else None))
        return (s, g) if grad else s

    def eval_fp64(self, pts, grad=False):
        """FP64 oracle (pi_fp64_eval_field): SingleEval in double at pts."""
        pts = np.ascontiguousarray(pts, dtype=np.float32)
        m = pts.shape[0]
        s = np.empty(m, np.float64)
        g = np.empty((m, 3), np.float64) if grad else None
        check(lib().pi_fp64_eval_field(self.h, ptr(pts, C.c_float), m, ptr(s, C.c_double),
                                       ptr(g, C.c_double) if grad else None))
        return (s, g) if grad else s

    def aniso_fp64(self):
        """FP64 oracle (pi_fp64_aniso): centres [n, 3], G [n, 3, 3], det [n], original order."""
        n = self.n
        xm = np.empty((n, 3), np.float64)
        g = np.empty((n, 3, 3), np.float64)
        d = np.empty(n, np.float64)
        check(lib().pi_fp64_aniso(self.h, ptr(xm, C.c_double), ptr(g, C.c_double), ptr(d, C.c_double)))
        return xm, g, d

    def scalars_fp64(self):
        o = np.empty(4, np.float64)
        check(lib().pi_fp64_scalars(self.h, ptr(o, C.c_double)))
        return dict(iso=o[0], max_scalar=o[1], influence2=o[2], sigma=o[3])

    def grid_dims(self):
        """UniformGrid lattice: dims (x, y, z), box (min/max per axis), point count."""
        dims = np.zeros(3, np.int32)
        box = np.zeros(6, np.float32)
        n = C.c_int64()
        check(lib().pi_grid_dims(self.h, ptr(dims, C.c_int32), ptr(box, C.c_float), C.byref(n)))
        return dims, box, n.value

    def grid_sample(self):
        """UniformGrid::gridSampling: values[dims z, y, x] (float32)."""
        dims, box, n = self.grid_dims()
        out = np.empty(n, np.float32)
        check(lib().pi_grid_sample(self.h, ptr(out, C.c_float), n))
        return out.reshape(int(dims[2]), int(dims[1]), int(dims[0]))

    def grid_sample_device(self, d_ptr, cap):
        check(lib().pi_grid_sample_device(self.h, C.c_void_p(d_ptr), cap))

    def write_ply(self, path):
        check(lib().pi_mesh_write_ply(self.h, path.encode()))

    def write_vti(self, path):
        check(lib().pi_grid_write_vti(self.h, path.encode()))

    def neighbors(self, pts):
        pts = np.ascontiguousarray(pts, dtype=np.float32)
        m = pts.shape[0]
        off = np.empty(m + 1, np.int64)
        tot = C.c_int64()
        rc = lib().pi_hashgrid_neighbors(self.h, ptr(pts, C.c_float), m, ptr(off, C.c_int64), None, 0,
                                         C.byref(tot))
        if rc not in (0, -5):
            check(rc)
        idx = np.empty(max(tot.value, 1), np.int32)
        check(lib().pi_hashgrid_neighbors(self.h, ptr(pts, C.c_float), m, ptr(off, C.c_int64),
                                          ptr(idx, C.c_int32), idx.shape[0], C.byref(tot)))
        return off, idx[:tot.value]

    def in_box(self, b1, b2):
        b1 = np.ascontiguousarray(b1, dtype=np.float32)
        b2 = np.ascontiguousarray(b2, dtype=np.float32)
        tot = C.c_int64()
        rc = lib().pi_hashgrid_in_box(self.h, ptr(b1, C.c_float), ptr(b2, C.c_float), None, 0, C.byref(tot))
        if rc not in (0, -5):
            check(rc)
        idx = np.empty(max(tot.value, 1), np.int32)
        check(lib().pi_hashgrid_in_box(self.h, ptr(b1, C.c_float), ptr(b2, C.c_float), ptr(idx, C.c_int32),
                                       idx.shape[0], C.byref(tot)))
        return idx[:tot.value]

    def dump(self, what):
        nb = C.c_size_t()
        check(lib().pi_stage_dump_size(self.h, what, C.byref(nb)))
        dtype, shape = {
            DUMP_KEYS: (np.int64, (-1,)), DUMP_INDEX_LIST: (np.int32, (-1,)),
            DUMP_CELL_OFFSETS: (np.int32, (-1,)), DUMP_XMEANS: (np.float32, (-1, 3)),
            DUMP_G: (np.float32, (-1, 3, 3)), DUMP_DET: (np.float32, (-1,)),
            DUMP_NORMALS: (np.float32, (-1, 3)), DUMP_NODES: (NODE_DTYPE, (-1,)),
            DUMP_FP64_FLAGS: (np.int8, (-1,)), DUMP_QEF_SAMPLES: (np.float32, (-1, 27)),
            DUMP_GRID_OF: (np.int32, (-1,)), DUMP_SPLASH: (np.int8, (-1,)),
            DUMP_VERTEX_EDGES: (np.int32, (-1, 2)),
        }[what]
        buf = np.empty(nb.value // np.dtype(dtype).itemsize, dtype)
        check(lib().pi_stage_dump(self.h, what, buf.ctypes.data_as(C.c_void_p), nb.value))
        return buf.reshape(shape)


def _declare_server(L):
    P = C.c_void_p
    sig = {
        "pi_server_create": (C.c_int, [C.c_int, C.c_int, C.c_size_t, C.POINTER(C.c_void_p)]),
        "pi_server_submit": (C.c_int, [P, C.POINTER(Params), C.POINTER(C.c_float), C.c_int64,
                                       C.POINTER(C.c_uint64)]),
        "pi_server_poll": (C.c_int, [P, C.c_uint64, C.POINTER(C.c_int)]),
        "pi_server_wait": (C.c_int, [P, C.c_uint64, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "pi_server_fetch": (C.c_int, [P, C.c_uint64, C.POINTER(C.c_float), C.POINTER(C.c_int32)]),
        "pi_server_stats": (C.c_int, [P] + [C.POINTER(C.c_int64)] * 5),
        "pi_server_submit_seq": (C.c_int, [P, C.POINTER(Params), C.POINTER(C.c_float), C.c_int64, C.c_uint64,
                                           C.POINTER(C.c_uint64)]),
        "pi_server_set_estimate": (C.c_int, [P, C.c_size_t, C.c_size_t]),
        "pi_server_info": (C.c_int, [P, C.POINTER(C.c_int64)]),
        "pi_server_destroy": (C.c_int, [P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


class Server:
    """pi_server: continuous batching of frame requests on one GPU."""

    def __init__(self, device=0, slots=8, budget_bytes=0):
        _declare_server(lib())
        h = C.c_void_p()
        check(lib().pi_server_create(device, slots, budget_bytes, C.byref(h)))
        self.h = h

    def submit(self, xyz, params, seq=0):
        xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        t = C.c_uint64()
        check(lib().pi_server_submit_seq(self.h, C.byref(params), ptr(xyz, C.c_float), xyz.shape[0], seq,
                                         C.byref(t)))
        return t.value

    def set_estimate(self, bytes_per_particle, fixed_bytes):
        check(lib().pi_server_set_estimate(self.h, bytes_per_particle, fixed_bytes))

    def info(self):
        out = (C.c_int64 * 8)()
        check(lib().pi_server_info(self.h, out))
        return dict(zip(["completed", "reserved_bytes", "resident_bytes", "resident_frames", "bypasses", "retries",
                         "resident_hits", "budget"], list(out)))

    def done(self, ticket):
        d = C.c_int()
        check(lib().pi_server_poll(self.h, ticket, C.byref(d)))
        return bool(d.value)

    def result(self, ticket):
        nv, nt = C.c_int64(), C.c_int64()
        lat, q = C.c_double(), C.c_double()
        check(lib().pi_server_wait(self.h, ticket, C.byref(nv), C.byref(nt), C.byref(lat), C.byref(q)))
        v = np.empty((nv.value, 3), np.float32)
        t = np.empty((nt.value, 3), np.int32)
        check(lib().pi_server_fetch(self.h, ticket, ptr(v, C.c_float), ptr(t, C.c_int32)))
        return v, t, lat.value, q.value

    def stats(self):
        vals = [C.c_int64() for _ in range(5)]
        check(lib().pi_server_stats(self.h, *[C.byref(x) for x in vals]))
        return dict(zip(["completed", "in_flight", "max_in_flight", "queued", "bytes_reserved"],
                        [x.value for x in vals]))

    def close(self):
        if self.h:
            lib().pi_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
