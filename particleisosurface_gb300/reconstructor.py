"""Python facade with the reference's class and method names.

    mesh = Mesh()
    rec = SurfReconstructor(particles, radiuses, mesh, radius)
    rec.Run(iso_factor, smooth_factor)          # src/surface_reconstructor.cpp:409
    writeObjFile(mesh, "frame.obj")              # src/main.cpp:54

Everything runs in the CUDA library through the C ABI (include/pisurf.h);
the facade only moves arrays.  Reference interfaces mirrored:
SurfReconstructor (include/surface_reconstructor.h:71-92), Evaluator
(include/evaluator.h:76-95), HashGrid (include/hash_grid.h:16-38),
MultiLevelSearcher (include/multi_level_researcher.h:8-40), Mesh
(include/global.h:86-115), and the run-mode switch IS_CONST_RADIUS
(include/iso_common.h:6): set it to False, as the reference's main does for
per-particle radii, and SurfReconstructor.Run uses `radiuses`.
"""
from __future__ import annotations

import numpy as np

from . import _native as N

_default_ctx = None

IS_CONST_RADIUS = True


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = N.Context(0)
    return _default_ctx


class Mesh:
    """Mesh container: vertices (float32 n x 3) and 1-based triangles, as the
    reference's Mesh::vertices / Mesh::tris; vertex_keys hold the leaf-id pair
    each vertex was inserted under (Mesh::insert_vert)."""

    def __init__(self, mesh_precision=10000):
        self.MESH_PRECISION = mesh_precision
        self.reset()

    def reset(self):
        self.vertices = np.zeros((0, 3), np.float32)
        self.tris = np.zeros((0, 3), np.int32)
        self.vertex_keys = np.zeros((0, 2), np.uint64)

    @property
    def verticesNum(self):
        return int(self.vertices.shape[0])

    @property
    def trianglesNum(self):
        return int(self.tris.shape[0])


def writeObjFile(mesh: Mesh, fn: str):
    """writeObjFile (src/main.cpp:54-67): "v %f %f %f" then "f %d %d %d"."""
    with open(fn, "w") as f:
        for p in mesh.vertices:
            f.write("v %f %f %f\n" % (p[0], p[1], p[2]))
        for t in mesh.tris:
            f.write("f %d %d %d\n" % (t[0], t[1], t[2]))


def writePlyFile(mesh: Mesh, fn: str):
    """writePlyFile (src/main.cpp:69-114): binary PLY, float32 vertices and
    0-based int face lists (mesh.tris are 1-based as in the reference)."""
    N.write_ply(fn, mesh.vertices, mesh.tris, one_based=True)


def readShonDyParticleData(file_name, is_const_radius=None):
    """readShonDyParticleData (src/main.cpp:281-327): "position" and, unless
    the radius is constant (IS_CONST_RADIUS by default), "particleRadius" of
    an HDF5 particle file, as float32 (positions [n, 3], radiuses [n] or
    empty).  The library reads the HDF5 format itself."""
    const = IS_CONST_RADIUS if is_const_radius is None else is_const_radius
    xyz, rad = N.load_hdf5(file_name, radius=not const)
    return xyz, (rad if rad is not None else np.zeros(0, np.float32))


def readShonDyParticleXDMF(dir_path, xdmf_file, target_frame=0):
    """readShonDyParticleXDMF (src/hdf5Utils.cpp:7-47): the frame files of
    an XDMF frame list, all or only frame target_frame (1-based)."""
    return N.load_xdmf(dir_path, xdmf_file, target_frame)


def loadParticlesFromCSV(csv_path, is_const_radius=True):
    """loadParticlesFromCSV (src/main.cpp:215-275): (particles [n, 3] float32,
    radiuses [n] float32, empty when is_const_radius)."""
    xyz, rad, _ = N.load_csv(csv_path, radius=not is_const_radius)
    return xyz, (rad if rad is not None else np.zeros(0, np.float32))


class HashGrid:
    def __init__(self, frame: N.Frame):
        self._f = frame
        info = frame.info()
        self.Bounding = np.array(info["bounding"], np.float32)
        self.CellSize = info["cell_size"]
        self.XYZCellNum = np.array(info["xyz_cell_num"], np.int64)
        self.CellNum = info["cell_num"]
        self.ParticlesNum = info["num_particles"]

    @property
    def IndexList(self):
        return self._f.dump(N.DUMP_INDEX_LIST)

    def GetPIdxList(self, pos):
        off, idx = self._f.neighbors(np.asarray(pos, np.float32).reshape(1, 3))
        return idx[off[0]:off[1]].tolist()

    def GetInBoxParticles(self, box1, box2):
        return self._f.in_box(box1, box2).tolist()


class Evaluator:
    def __init__(self, frame: N.Frame):
        self._f = frame

    def SingleEval(self, pos):
        return float(self._f.eval(np.asarray(pos, np.float32).reshape(1, 3))[0])

    def SingleEvalWithGrad(self, pos):
        s, g = self._f.eval(np.asarray(pos, np.float32).reshape(1, 3), grad=True)
        return float(s[0]), g[0]

    def eval_many(self, pts, grad=False):
        return self._f.eval(pts, grad=grad)

    def getIsoValue(self):
        return self._f.info()["iso_value"]

    def getMaxScalar(self):
        return self._f.info()["max_scalar"]

    @property
    def GlobalxMeans(self):
        return self._f.dump(N.DUMP_XMEANS)

    @property
    def GlobalGs(self):
        return self._f.dump(N.DUMP_G)

    @property
    def GlobalDeterminant(self):
        return self._f.dump(N.DUMP_DET)

    @property
    def PariclesNormals(self):
        return self._f.dump(N.DUMP_NORMALS)


class MultiLevelSearcher:
    """The radius bins of a frame with per-particle radii
    (src/multi_level_reseacher.cpp): one hash grid per non-empty bin."""

    def __init__(self, frame):
        self._f = frame
        info = frame.info()
        self._min, self._max, self._n = info["radius_min"], info["radius_max"], info["num_particles"]
        self._grids = [frame.grid(k) for k in range(info["num_grids"])]

    def getMinRadius(self):
        return self._min

    def getMaxRadius(self):
        return self._max

    def getParticlesNum(self):
        return self._n

    def getSearchers(self):
        """One record per bin grid: bounding, dims, cell_size, count, radius_id."""
        return self._grids

    def GetNeighbors(self, pos):
        """GetNeighbors (src/multi_level_reseacher.cpp:79-92)."""
        off, idx = self._f.neighbors(np.asarray(pos, np.float32).reshape(1, 3))
        return idx.tolist()


class SurfReconstructor:
    def __init__(self, particles, radiuses, mesh: Mesh, radius: float, ctx: N.Context | None = None,
                 qef: bool = False, splash: bool = False):
        self._particles = np.ascontiguousarray(np.asarray(particles, np.float32).reshape(-1, 3))
        self._radiuses = np.ascontiguousarray(np.asarray(radiuses, np.float32).reshape(-1))
        self._radius = float(radius)
        self._mesh = mesh
        self._ctx = ctx or default_context()
        self._qef = qef
        self._splash = splash
        self._frame = None
        self._var_r = False

    def Run(self, iso_factor=1.9, smooth_factor=2.0):
        self._mesh.reset()
        var_r = not IS_CONST_RADIUS
        radius = float(self._radiuses.min()) if var_r and self._radiuses.size else self._radius
        params = N.default_params(radius, smooth_factor=smooth_factor, iso_factor=iso_factor, qef=self._qef,
                                  splash=self._splash)
        f = N.Frame(self._ctx, params).upload(self._particles)
        if var_r:
            f.upload_radii(self._radiuses)
        self._var_r = var_r
        self._frame = f.run()
        v, t, k = self._frame.mesh(keys=True)
        self._mesh.vertices = v
        self._mesh.tris = t + 1
        self._mesh.vertex_keys = k

    def _info(self):
        return self._frame.info()

    def getDepthMax(self):
        return self._info()["depth_max"]

    def getDepthMin(self):
        return self._info()["depth_min"]

    def getOverSampleQEF(self):
        return 2

    def getConstRadius(self):
        return self._radius

    def getGlobalParticlesNum(self):
        return int(self._particles.shape[0])

    def getGlobalParticles(self):
        return self._particles

    def getHashGrid(self):
        return None if self._var_r else HashGrid(self._frame)

    def getSearcher(self):
        return MultiLevelSearcher(self._frame) if self._var_r else None

    def getEvaluator(self):
        return Evaluator(self._frame)

    def getRoot(self):
        """All octree nodes (pi_node records, creation order); node 0 is the root."""
        return self._frame.dump(N.DUMP_NODES)

    def frame_info(self):
        return self._info()


class UniformGrid:
    """UniformGrid (include/marching.h:18-70, src/marching.cpp), constant
    radius: Run samples the field on the lattice of spacing r over the
    particles' box (resizeRootBoxConstR) and writes it as a VTK image
    <filepath>/<filename>.vti; the values stay in `_Scalars` (x fastest, as
    the reference stores them) and `dims`, `steps`, `_BoundingBox` describe
    the lattice."""

    def __init__(self, particles, radius, ctx: N.Context | None = None):
        self._GlobalParticles = np.ascontiguousarray(np.asarray(particles, np.float32).reshape(-1, 3))
        self._GlobalParticlesNum = int(self._GlobalParticles.shape[0])
        self._RADIUS = float(radius)
        self._ctx = ctx or default_context()
        self._SMOOTH_FACTOR = 2.0
        self._frame = None
        self.dims = np.zeros(3, np.int32)
        self.steps = np.zeros(3, np.int32)
        self._BoundingBox = np.zeros(6, np.float32)
        self._Scalars = np.zeros(0, np.float32)

    def Run(self, iso_value=0.0, filename=None, filepath="."):
        """The reference computes its own iso value (RecommendIsoValueConstR)
        and ignores iso_value, as here."""
        params = N.default_params(self._RADIUS, smooth_factor=self._SMOOTH_FACTOR)
        self._frame = N.Frame(self._ctx, params).upload(self._GlobalParticles)
        self._frame.hashgrid().aniso().normals()
        dims, box, _ = self._frame.grid_dims()
        self.dims = dims
        self.steps = dims - 1
        self._BoundingBox = box
        self._Scalars = self._frame.grid_sample().ravel()
        if filename:
            import os
            self._frame.write_vti(os.path.join(filepath, filename + ".vti"))
        return self._Scalars

    def getIsoValue(self):
        return self._frame.info()["iso_value"]

    def getMaxScalar(self):
        return self._frame.info()["max_scalar"]
