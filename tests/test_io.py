"""Host data formats (no GPU): the CSV particle loader against a restatement
of the reference's loadParticlesFromCSV (src/main.cpp:215-275), and the
binary PLY writer against the file RPly writes for writePlyFile
(src/main.cpp:69-114)."""
import re
import struct

import numpy as np
import pytest

from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B


@pytest.fixture(scope="module", autouse=True)
def _lib():
    B.build()


AXES = [r"^(.*(:|_|-)( *)(x|0)(\"*)|x)$", r"^(.*(:|_|-)( *)(y|1)(\"*)|y)$", r"^(.*(:|_|-)( *)(z|2)(\"*)|z)$"]
RAD = r"^((.*)radius|r)$"


def ref_columns(header, want_radius):
    titles = header.replace('"', "").split(",")
    if titles and titles[-1] == "":
        titles = titles[:-1]

    def first(p):
        for i, t in enumerate(titles):
            if re.fullmatch(p, t, re.IGNORECASE):
                return i
        return len(titles)

    return [first(p) for p in AXES] + ([first(RAD)] if want_radius else [-1])


@pytest.mark.parametrize("header", [
    '"Points:0","Points:1","Points:2","radius"',
    "id,pos_x,pos_y,pos_z,particle_radius",
    "X,Y,Z,R",
    "vel-x,vel-y,vel-z,density,r",
    "p_0,p_ 1,p_2,Radius",
])
def test_csv_columns_and_values(tmp_path, header):
    rng = np.random.default_rng(abs(hash(header)) % 1000)
    cols = ref_columns(header, True)
    ncol = len(header.split(","))
    rows = rng.normal(0, 1, (50, ncol)).astype(np.float32)
    text = header + "\n" + "\n".join(",".join("%.9g" % v for v in r) for r in rows) + "\n\n1,2,3\n"
    path = tmp_path / "p.csv"
    path.write_text(text)
    xyz, rad, got = N.load_csv(path, radius=True)
    assert list(got) == cols
    np.testing.assert_array_equal(xyz, rows[:, cols[:3]])
    np.testing.assert_array_equal(rad, rows[:, cols[3]])
    # rows stop at the first empty line, as the reference's loop does
    assert xyz.shape[0] == 50


def test_csv_errors(tmp_path):
    p = tmp_path / "bad.csv"
    p.write_text("a,b,c\n1,2,3\n")
    with pytest.raises(N.PiError) as e:
        N.load_csv(p)
    assert e.value.code == N.PI_ERR_INVALID
    p.write_text("x,y,z\n1,2,abc\n")
    with pytest.raises(N.PiError) as e:
        N.load_csv(p)
    assert e.value.code == N.PI_ERR_INVALID


def test_ply_bytes(tmp_path):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    t = np.array([[1, 2, 3], [1, 3, 4]], np.int32)  # 1-based, as Mesh::tris
    path = tmp_path / "m.ply"
    N.write_ply(path, v, t, one_based=True)
    raw = path.read_bytes()
    head = (b"ply\nformat binary_little_endian 1.0\nelement vertex 4\nproperty float32 x\n"
            b"property float32 y\nproperty float32 z\nelement face 2\n"
            b"property list uchar int vertex_indices\nend_header\n")
    assert raw.startswith(head)
    body = raw[len(head):]
    assert body[:48] == v.astype("<f4").tobytes()
    faces = body[48:]
    assert len(faces) == 2 * 13
    for k, tri in enumerate(t):
        assert faces[13 * k] == 3
        assert struct.unpack("<3i", faces[13 * k + 1:13 * k + 13]) == tuple(int(x) - 1 for x in tri)
