"""A small HDF5 writer for test fixtures: particle files as the reference's
readShonDyParticleData reads them (a flat "position" dataset of 3N values and
an optional "particleRadius" of N values in the root group).  Written from
the HDF5 File Format Specification (version 3.0); it emits the structures the
library's reader handles, in two families:

  layout="v0": superblock version 0, a root group with a symbol table
    (version 1 B-tree, one symbol node, local heap of names), version 1
    object headers; datasets contiguous, chunked (version 1 B-tree of chunks,
    optional shuffle + deflate filters) or compact.
  layout="v2": superblock version 2, version 2 object headers ("OHDR", with
    Jenkins lookup3 checksums), a compact root group of link messages.

The writer is test infrastructure; the reader under test is the library's
(particleisosurface_gb300/csrc/h5.cu)."""
import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIG = b"\x89HDF\r\n\x1a\n"


def lookup3(data, initval=0):
    """Bob Jenkins' lookup3 hashlittle (public domain), the checksum of
    version 2 HDF5 metadata."""
    def rot(x, k):
        return ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF

    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & 0xFFFFFFFF
    i = 0
    while n > 12:
        a = (a + int.from_bytes(data[i:i + 4], "little")) & 0xFFFFFFFF
        b = (b + int.from_bytes(data[i + 4:i + 8], "little")) & 0xFFFFFFFF
        c = (c + int.from_bytes(data[i + 8:i + 12], "little")) & 0xFFFFFFFF
        a = (a - c) & 0xFFFFFFFF; a ^= rot(c, 4); c = (c + b) & 0xFFFFFFFF
        b = (b - a) & 0xFFFFFFFF; b ^= rot(a, 6); a = (a + c) & 0xFFFFFFFF
        c = (c - b) & 0xFFFFFFFF; c ^= rot(b, 8); b = (b + a) & 0xFFFFFFFF
        a = (a - c) & 0xFFFFFFFF; a ^= rot(c, 16); c = (c + b) & 0xFFFFFFFF
        b = (b - a) & 0xFFFFFFFF; b ^= rot(a, 19); a = (a + c) & 0xFFFFFFFF
        c = (c - b) & 0xFFFFFFFF; c ^= rot(b, 4); b = (b + a) & 0xFFFFFFFF
        n -= 12
        i += 12
    if n == 0:
        return c
    tail = data[i:] + b"\0" * (12 - n)
    a = (a + int.from_bytes(tail[0:4], "little")) & 0xFFFFFFFF
    b = (b + int.from_bytes(tail[4:8], "little")) & 0xFFFFFFFF
    c = (c + int.from_bytes(tail[8:12], "little")) & 0xFFFFFFFF
    c ^= b; c = (c - rot(b, 14)) & 0xFFFFFFFF
    a ^= c; a = (a - rot(c, 11)) & 0xFFFFFFFF
    b ^= a; b = (b - rot(a, 25)) & 0xFFFFFFFF
    c ^= b; c = (c - rot(b, 16)) & 0xFFFFFFFF
    a ^= c; a = (a - rot(c, 4)) & 0xFFFFFFFF
    b ^= a; b = (b - rot(a, 14)) & 0xFFFFFFFF
    c ^= b; c = (c - rot(b, 24)) & 0xFFFFFFFF
    return c


def _pad8(b):
    return b + b"\0" * (-len(b) % 8)


def _dtype_msg(dt):
    """Datatype message: IEEE float of the array's size and byte order."""
    big = dt.byteorder == ">"
    if dt.itemsize == 8:
        props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
        sign = 63
    else:
        props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
        sign = 31
    return bytes([0x11, 0x20 | (1 if big else 0), sign, 0]) + struct.pack("<I", dt.itemsize) + props


class _File:
    def __init__(self):
        self.buf = bytearray()

    def alloc(self, data, align=8):
        self.buf += b"\0" * (-len(self.buf) % align)
        off = len(self.buf)
        self.buf += data
        return off

    def put(self, off, data):
        self.buf[off:off + len(data)] = data


def _dataset_v0(f, arr, storage, chunk, filters, base):
    """Raw data and the messages of a version 1 object header for arr."""
    dt = arr.dtype
    raw = arr.tobytes()
    n = arr.size
    msgs = [(0x0001, struct.pack("<BBBB4x", 1, 1, 0, 0) + struct.pack("<Q", n)), (0x0003, _dtype_msg(dt))]
    if storage == "contiguous":
        addr = f.alloc(raw) - base
        msgs.append((0x0008, struct.pack("<BBQQ", 3, 1, addr, len(raw))))
    elif storage == "compact":
        msgs.append((0x0008, struct.pack("<BBH", 3, 0, len(raw)) + raw))
    else:  # chunked, one B-tree leaf node
        es = dt.itemsize
        keys = []
        for s in range(0, n, chunk):
            piece = arr[s:s + chunk]
            if len(piece) < chunk:
                piece = np.concatenate([piece, np.zeros(chunk - len(piece), dt)]).astype(dt)
            data = piece.tobytes()
            if "shuffle" in filters:
                data = np.frombuffer(data, np.uint8).reshape(chunk, es).T.tobytes()
            if "deflate" in filters:
                data = zlib.compress(data, 6)
            keys.append((len(data), s, f.alloc(data) - base))
        node = bytearray(b"TREE" + bytes([1, 0]) + struct.pack("<HQQ", len(keys), UNDEF, UNDEF))
        for size, s, a in keys:
            node += struct.pack("<IIQQQ", size, 0, s, 0, a)
        node += struct.pack("<IIQQ", 0, 0, n, 0)
        tree = f.alloc(bytes(node)) - base
        msgs.append((0x0008, struct.pack("<BBBQ", 3, 2, 2, tree) + struct.pack("<II", chunk, es)))
        if filters:
            fl = struct.pack("<BB6x", 1, len(filters))
            for name in filters:
                if name == "shuffle":
                    fl += struct.pack("<HHHHI", 2, 0, 1, 1, es) + b"\0" * 4
                else:
                    fl += struct.pack("<HHHHI", 1, 0, 0, 1, 6) + b"\0" * 4
            msgs.append((0x000B, fl))
    return msgs


def _ohdr_v1(f, msgs):
    body = b""
    for t, d in msgs:
        d = _pad8(d)
        body += struct.pack("<HHB3x", t, len(d), 0) + d
    head = struct.pack("<BBHII", 1, 0, len(msgs), 1, len(body)) + b"\0" * 4
    return f.alloc(head + body)


def _ohdr_v2(f, msgs):
    body = b""
    for t, d in msgs:
        body += struct.pack("<BHB", t, len(d), 0) + d
    head = b"OHDR" + bytes([2, 1]) + struct.pack("<H", len(body))
    blob = head + body
    return f.alloc(blob + struct.pack("<I", lookup3(blob)))


def write_particles(path, position, radius=None, layout="v0", storage="contiguous", chunk=1024, filters=(),
                    dtype="<f8", userblock=0):
    """position: (N, 3) array written flat (3N values); radius: (N,) or None."""
    datasets = {"position": np.ascontiguousarray(position, np.float64).reshape(-1).astype(dtype)}
    if radius is not None:
        datasets["particleRadius"] = np.ascontiguousarray(radius, np.float64).reshape(-1).astype(dtype)
    f = _File()
    f.buf += b"\0" * userblock
    if layout == "v0":
        sb = f.alloc(b"\0" * 96)
        names = sorted(datasets)
        heap_data = b"\0" * 8
        offs = {}
        for nm in names:
            offs[nm] = len(heap_data)
            heap_data += _pad8(nm.encode() + b"\0")
        heap_seg = f.alloc(heap_data)
        heap = f.alloc(b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap_data), UNDEF, heap_seg - userblock))
        objs = {nm: _ohdr_v1(f, _dataset_v0(f, datasets[nm], storage, chunk, filters, userblock)) for nm in names}
        snod = bytearray(b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(names)))
        for nm in names:
            snod += struct.pack("<QQII16x", offs[nm], objs[nm] - userblock, 0, 0)
        snod += b"\0" * (40 * (8 - len(names)))
        snod_at = f.alloc(bytes(snod))
        tree = f.alloc(b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", 1, UNDEF, UNDEF) +
                       struct.pack("<QQQ", 0, snod_at - userblock, offs[names[-1]]))
        root = _ohdr_v1(f, [(0x0011, struct.pack("<QQ", tree - userblock, heap - userblock))])
        s = bytearray(SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0))
        s += struct.pack("<QQQQ", userblock, UNDEF, len(f.buf) - userblock, UNDEF)
        s += struct.pack("<QQII", 0, root - userblock, 1, 0) + struct.pack("<QQ", tree - userblock, heap - userblock)
        f.put(sb, bytes(s))
    else:
        sb = f.alloc(b"\0" * 48)
        links = []
        for nm, arr in datasets.items():
            raw = arr.tobytes()
            space = struct.pack("<BBBB", 2, 1, 0, 1) + struct.pack("<Q", arr.size)
            if storage == "compact":
                lay = struct.pack("<BBH", 3, 0, len(raw)) + raw
            else:
                lay = struct.pack("<BBQQ", 3, 1, f.alloc(raw) - userblock, len(raw))
            oh = _ohdr_v2(f, [(0x01, space), (0x03, _dtype_msg(arr.dtype)), (0x08, lay)])
            links.append((0x06, bytes([1, 0, len(nm)]) + nm.encode() + struct.pack("<Q", oh - userblock)))
        root = _ohdr_v2(f, links)
        s = SIG + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", userblock, UNDEF, len(f.buf) - userblock, root - userblock)
        f.put(sb, s + struct.pack("<I", lookup3(s)))
    with open(path, "wb") as fh:
        fh.write(bytes(f.buf))
