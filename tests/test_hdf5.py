"""CPU tests of the library's HDF5 particle reader and XDMF frame list
(pi_load_hdf5, pi_hdf5_dataset, pi_load_xdmf; the reference's
readShonDyParticleData, src/main.cpp:281-327, and readShonDyParticleXDMF,
src/hdf5Utils.cpp:7-47).  No GPU is needed.

Pins: a file written by the HDF5 library itself (a MATLAB 7.3 file of SciPy's
test data: 512-byte user block, superblock version 0, symbol-table group),
read to its known values; and files of every structure the reader handles,
written by tests/h5write.py from the format specification, read back bit for
bit (each double rounded to float as the reference's Eigen::Vector3f(double,
...) and float(double) do)."""
import os

import numpy as np
import pytest

import h5write as W
from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B
from particleisosurface_gb300 import reconstructor as R


@pytest.fixture(scope="module", autouse=True)
def _lib():
    B.build()


def _scipy_hdf5_mat():
    try:
        import scipy.io.matlab as m
    except Exception:
        return None
    p = os.path.join(os.path.dirname(m.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    return p if os.path.exists(p) else None


def test_reads_a_file_written_by_the_hdf5_library():
    p = _scipy_hdf5_mat()
    if p is None:
        pytest.skip("SciPy's HDF5 MAT test file is not installed")
    a = N.hdf5_dataset(p, "testdouble")
    # MATLAB's 1 x 9 row pi / 4 * (0:8), stored column-major as 9 x 1
    assert a.shape == (9, 1)
    np.testing.assert_array_equal(a.ravel(), np.pi / 4 * np.arange(9))


VARIANTS = [
    dict(),
    dict(userblock=512),
    dict(storage="compact"),
    dict(storage="chunked", chunk=256),
    dict(storage="chunked", chunk=300, filters=("shuffle", "deflate")),
    dict(storage="chunked", chunk=4096, filters=("deflate",), dtype=">f8"),
    dict(dtype="<f4"),
    dict(layout="v2"),
    dict(layout="v2", storage="compact", dtype=">f4"),
]


@pytest.mark.parametrize("kw", VARIANTS, ids=[",".join("%s=%s" % i for i in v.items()) or "v0" for v in VARIANTS])
def test_particle_file_round_trip(tmp_path, kw):
    rng = np.random.default_rng(7)
    pos = rng.normal(0.0, 1.0, size=(2000, 3)) * 0.37 + 1.5
    rad = rng.uniform(0.005, 0.02, 2000)
    p = tmp_path / "frame.h5"
    W.write_particles(p, pos, rad, **kw)
    dt = np.dtype(kw.get("dtype", "<f8"))
    xyz, r = N.load_hdf5(p, radius=True)
    np.testing.assert_array_equal(xyz, pos.astype(dt).astype(np.float64).astype(np.float32))
    np.testing.assert_array_equal(r, rad.astype(dt).astype(np.float64).astype(np.float32))
    xyz2, r2 = N.load_hdf5(p)
    assert r2 is None
    np.testing.assert_array_equal(xyz2, xyz)
    flat = N.hdf5_dataset(p, "position")
    assert flat.shape == (6000,)
    # the facade: radii only with per-particle radii
    xf, rf = R.readShonDyParticleData(str(p))
    np.testing.assert_array_equal(xf, xyz)
    assert rf.size == 0
    xf, rf = R.readShonDyParticleData(str(p), is_const_radius=False)
    np.testing.assert_array_equal(rf, r)


def test_particle_file_errors(tmp_path):
    rng = np.random.default_rng(8)
    pos = rng.normal(size=(100, 3))
    p = tmp_path / "nr.h5"
    W.write_particles(p, pos)  # no particleRadius
    with pytest.raises(N.PiError) as e:
        N.load_hdf5(p, radius=True)
    assert e.value.code == N.PI_ERR_INVALID and "particleRadius" in str(e.value)
    with pytest.raises(N.PiError) as e:
        N.load_hdf5(tmp_path / "missing.h5")
    assert e.value.code == N.PI_ERR_INVALID
    bad = tmp_path / "bad.h5"
    bad.write_bytes(b"not an hdf5 file" * 100)
    with pytest.raises(N.PiError) as e:
        N.load_hdf5(bad)
    assert e.value.code == N.PI_ERR_INVALID and "HDF5" in str(e.value)
    # a short buffer: PI_ERR_LIMIT with the count reported
    import ctypes as C
    n = C.c_int64()
    buf = np.zeros((10, 3), np.float32)
    rc = N.lib().pi_load_hdf5(str(p).encode(), N.ptr(buf, C.c_float), None, 10, C.byref(n))
    assert rc == N.PI_ERR_LIMIT and n.value == 100


XDMF = """<?xml version="1.0" ?>
<!DOCTYPE Xdmf SYSTEM "Xdmf.dtd" []>
<Xdmf Version="2.0">
  <!-- three frames -->
  <Domain Name="ShonDy">
    <Grid Name="TimeSeries" GridType="Collection" CollectionType="Temporal">
      <Grid Name="p0" GridType="Uniform">
        <Time Value="0.0"/>
        <Geometry GeometryType="XYZ"><DataItem Dimensions="30 3" Format="HDF">frame_0.h5:/position</DataItem></Geometry>
      </Grid>
      <Grid Name="p1" GridType="Uniform">
        <Geometry GeometryType="XYZ"><DataItem Format="HDF"><![CDATA[frame_1.h5:/position]]></DataItem></Geometry>
      </Grid>
      <Grid Name="p2">
        <Geometry><DataItem Format="HDF">a&amp;b.h5:/position</DataItem></Geometry>
      </Grid>
    </Grid>
  </Domain>
</Xdmf>
"""


def test_xdmf_frame_list(tmp_path):
    (tmp_path / "series.xdmf").write_text(XDMF)
    assert N.load_xdmf(tmp_path, "series.xdmf") == ["frame_0.h5", "frame_1.h5", "a&b.h5"]
    assert N.load_xdmf(tmp_path, "series.xdmf", 2) == ["frame_1.h5"]
    # out of range: every frame (src/hdf5Utils.cpp:33-44)
    assert N.load_xdmf(tmp_path, "series.xdmf", 9) == ["frame_0.h5", "frame_1.h5", "a&b.h5"]
    assert R.readShonDyParticleXDMF(str(tmp_path), "series.xdmf", 3) == ["a&b.h5"]
    with pytest.raises(N.PiError) as e:
        N.load_xdmf(tmp_path, "none.xdmf")
    assert e.value.code == N.PI_ERR_INVALID
    (tmp_path / "bad.xdmf").write_text("<Xdmf><Domain></Xdmf>")
    with pytest.raises(N.PiError):
        N.load_xdmf(tmp_path, "bad.xdmf")


def test_hdf5_frame_list_end_to_end(tmp_path):
    """An XDMF list of HDF5 frames, each read as the reference's frame loop
    reads it (src/main.cpp:336-351)."""
    rng = np.random.default_rng(9)
    frames = []
    for k in range(2):
        pos = rng.normal(size=(500 + k, 3))
        W.write_particles(tmp_path / ("frame_%d.h5" % k), pos, layout="v2" if k else "v0")
        frames.append(pos)
    (tmp_path / "series.xdmf").write_text(XDMF)
    names = N.load_xdmf(tmp_path, "series.xdmf")[:2]
    for name, pos in zip(names, frames):
        xyz, _ = N.load_hdf5(tmp_path / name)
        np.testing.assert_array_equal(xyz, pos.astype(np.float32))
