"""A minimal HDF5 writer and reader for snapshot files (no HDF5 library is needed).

Flou writes its snapshots as VTKHDF files through HDF5.jl (src/FlouSpatial/IO.jl:16-126,
src/FlouBiz/FlouBiz.jl:38-113): one group tree of contiguous datasets plus two attributes.
This module encodes exactly that subset of the HDF5 file format (format specification 3.0):

- superblock version 2 (8-byte offsets and lengths), with its checksum;
- version-2 object headers ("OHDR", one chunk, checksummed) for every group and dataset;
- groups in the compact "new-style" form: a Link Info message (no fractal heap, no B-tree), a
  Group Info message and one hard-link message per member;
- datasets with a version-2 dataspace (scalar or simple), a version-1 datatype (IEEE float64,
  little-endian signed / unsigned integers, fixed-length ASCII strings), a version-3 fill-value
  message and a version-3 contiguous layout message, raw data right after the header;
- attributes as version-3 attribute messages in the object header.

Checksums are Bob Jenkins' lookup3 `hashlittle` with initial value 0, as HDF5 uses.
A tree is a dict: a numpy array is a dataset, a dict a group, and the key "@attrs" of a group
or the pair (array, {name: value}) of a dataset carries attributes; an attribute value is a
numpy array or a `bytes` string.
"""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"


# ---------------------------------------------------------------------------------------
# lookup3 (Bob Jenkins, 2006, public domain), byte-wise little-endian form
# ---------------------------------------------------------------------------------------
def _rot(x, k):
    return ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF


def lookup3(data, initval=0):
    """hashlittle(data, len(data), initval) of lookup3.c."""
    M = 0xFFFFFFFF
    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & M
    k = bytes(data)
    i = 0
    while n > 12:
        a = (a + int.from_bytes(k[i:i + 4], "little")) & M
        b = (b + int.from_bytes(k[i + 4:i + 8], "little")) & M
        c = (c + int.from_bytes(k[i + 8:i + 12], "little")) & M
        a = (a - c) & M; a ^= _rot(c, 4); c = (c + b) & M
        b = (b - a) & M; b ^= _rot(a, 6); a = (a + c) & M
        c = (c - b) & M; c ^= _rot(b, 8); b = (b + a) & M
        a = (a - c) & M; a ^= _rot(c, 16); c = (c + b) & M
        b = (b - a) & M; b ^= _rot(a, 19); a = (a + c) & M
        c = (c - b) & M; c ^= _rot(b, 4); b = (b + a) & M
        n -= 12
        i += 12
    if n == 0:
        return c
    tail = k[i:i + n] + b"\0" * (12 - n)
    a = (a + int.from_bytes(tail[0:4], "little")) & M
    b = (b + int.from_bytes(tail[4:8], "little")) & M
    c = (c + int.from_bytes(tail[8:12], "little")) & M
    c ^= b; c = (c - _rot(b, 14)) & M
    a ^= c; a = (a - _rot(c, 11)) & M
    b ^= a; b = (b - _rot(a, 25)) & M
    c ^= b; c = (c - _rot(b, 16)) & M
    a ^= c; a = (a - _rot(c, 4)) & M
    b ^= a; b = (b - _rot(a, 14)) & M
    c ^= b; c = (c - _rot(b, 24)) & M
    return c


# ---------------------------------------------------------------------------------------
# messages
# ---------------------------------------------------------------------------------------
def _datatype(arr):
    """(datatype message bytes, element size) of a numpy dtype or a bytes string."""
    if isinstance(arr, bytes):   # fixed-length ASCII, null-terminated padding
        return bytes([0x13, 0x00, 0x00, 0x00]) + struct.pack("<I", len(arr)), len(arr)
    dt = np.dtype(arr.dtype)
    if dt == np.float64:
        return (bytes([0x11, 0x20, 0x3F, 0x00]) + struct.pack("<I", 8) +
                struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)), 8
    if dt.kind in "iu":
        bits = 0x08 if dt.kind == "i" else 0x00
        return bytes([0x10, bits, 0x00, 0x00]) + struct.pack("<I", dt.itemsize) + \
            struct.pack("<HH", 0, 8 * dt.itemsize), dt.itemsize
    raise TypeError("unsupported dataset type %s" % dt)


def _dataspace(shape):
    if shape is None:   # scalar
        return bytes([2, 0, 0, 0])
    return bytes([2, len(shape), 0, 1]) + b"".join(struct.pack("<Q", int(d)) for d in shape)


def _payload(value):
    """(shape or None for a scalar, raw little-endian bytes) of an attribute or dataset value."""
    if isinstance(value, bytes):
        return None, value
    a = np.ascontiguousarray(value)
    if a.dtype.kind == "f":
        a = a.astype("<f8")
    elif a.dtype.kind in "iu":
        a = a.astype(a.dtype.newbyteorder("<"))
    return a.shape, a.tobytes()


def _message(mtype, body):
    return struct.pack("<BHB", mtype, len(body), 0) + body


def _attribute(name, value):
    dt, _ = _datatype(value if isinstance(value, bytes) else np.asarray(value))
    shape, raw = _payload(value)
    ds = _dataspace(shape)
    nm = name.encode("ascii") + b"\0"
    body = struct.pack("<BBHHHB", 3, 0, len(nm), len(dt), len(ds), 0) + nm + dt + ds + raw
    return _message(12, body)


def _object_header(messages):
    chunk = b"".join(messages)
    head = b"OHDR" + bytes([2, 0x02]) + struct.pack("<I", len(chunk)) + chunk
    return head + struct.pack("<I", lookup3(head))


# ---------------------------------------------------------------------------------------
# writer
# ---------------------------------------------------------------------------------------
def _split(node):
    """(kind, payload, attrs): kind 'group' (dict of members) or 'dataset' (array)."""
    if isinstance(node, dict):
        attrs = node.get("@attrs", {})
        return "group", {k: v for k, v in node.items() if k != "@attrs"}, attrs
    if isinstance(node, tuple):
        return "dataset", np.asarray(node[0]), node[1]
    return "dataset", np.asarray(node), {}


def _header_size(node):
    """Size of a node's object header (it does not depend on any address)."""
    kind, payload, attrs = _split(node)
    if kind == "group":
        msgs = [_message(2, bytes(18)), _message(10, bytes(2))]
        msgs += [_message(6, bytes(3 + len(k.encode("ascii")) + 8)) for k in payload]
    else:
        dt, _ = _datatype(payload)
        msgs = [_message(1, _dataspace(payload.shape)), _message(3, dt), _message(5, bytes(2)),
                _message(8, bytes(18))]
    msgs += [_attribute(k, v) for k, v in attrs.items()]
    return len(_object_header(msgs))


def write(path, tree):
    """Writes `tree` (the root group) to an HDF5 file at `path`."""
    # pass 1: addresses (depth first: a node's header, then its raw data, then its members)
    order = []
    addr = {}
    pos = [48]

    def place(node, key):
        kind, payload, _ = _split(node)
        addr[key] = pos[0]
        pos[0] += _header_size(node)
        order.append((key, node))
        if kind == "dataset":
            addr[key + ("@data",)] = pos[0]
            pos[0] += payload.nbytes
        else:
            for name, child in payload.items():
                place(child, key + (name,))

    place(tree, ())
    eof = pos[0]
    # pass 2: bytes
    out = bytearray(eof)
    sb = SIGNATURE + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", 0, UNDEF, eof, addr[()])
    out[0:48] = sb + struct.pack("<I", lookup3(sb))
    for key, node in order:
        kind, payload, attrs = _split(node)
        if kind == "group":
            msgs = [_message(2, bytes([0, 0]) + struct.pack("<QQ", UNDEF, UNDEF)), _message(10, bytes([0, 0]))]
            for name in payload:
                nm = name.encode("ascii")
                if not 0 < len(nm) < 256:
                    raise ValueError("link names must be 1 to 255 ASCII bytes")
                msgs.append(_message(6, bytes([1, 0, len(nm)]) + nm + struct.pack("<Q", addr[key + (name,)])))
        else:
            dt, _ = _datatype(payload)
            shape, raw = _payload(payload)
            msgs = [_message(1, _dataspace(shape)), _message(3, dt), _message(5, bytes([3, 0x09])),
                    _message(8, bytes([3, 1]) + struct.pack("<QQ", addr[key + ("@data",)], len(raw)))]
            a = addr[key + ("@data",)]
            out[a:a + len(raw)] = raw
        msgs += [_attribute(k, v) for k, v in attrs.items()]
        h = _object_header(msgs)
        out[addr[key]:addr[key] + len(h)] = h
    with open(path, "wb") as f:
        f.write(bytes(out))


# ---------------------------------------------------------------------------------------
# reader (the subset above; checks every checksum)
# ---------------------------------------------------------------------------------------
def _parse_datatype(b):
    cls, ver = b[0] & 0x0F, b[0] >> 4
    size = struct.unpack_from("<I", b, 4)[0]
    if ver != 1:
        raise ValueError("datatype version %d" % ver)
    if cls == 1 and size == 8:
        return np.dtype("<f8"), 20
    if cls == 0:
        return np.dtype(("<i%d" if b[1] & 0x08 else "<u%d") % size), 12
    if cls == 3:
        return ("S", size), 8
    raise ValueError("unsupported datatype class %d" % cls)


def _parse_dataspace(b):
    if b[0] != 2:
        raise ValueError("dataspace version %d" % b[0])
    rank, typ = b[1], b[3]
    if typ == 0:
        return None, 4
    dims = struct.unpack_from("<%dQ" % rank, b, 4)
    return tuple(dims), 4 + 8 * rank * (2 if b[2] & 1 else 1)


def _decode(dtype, shape, raw):
    if isinstance(dtype, tuple):
        return bytes(raw)
    a = np.frombuffer(bytes(raw), dtype=dtype)
    return a.reshape(shape) if shape is not None else a[0]


def read(path):
    """The tree of an HDF5 file written by `write`: groups as dicts (attributes under "@attrs"),
    datasets as numpy arrays (their attributes are not returned)."""
    buf = open(path, "rb").read()
    if buf[:8] != SIGNATURE or buf[8] != 2:
        raise ValueError("%s: not an HDF5 file with a version-2 superblock" % path)
    if struct.unpack_from("<I", buf, 44)[0] != lookup3(buf[:44]):
        raise ValueError("%s: superblock checksum mismatch" % path)
    root = struct.unpack_from("<Q", buf, 36)[0]

    def node(at):
        if buf[at:at + 4] != b"OHDR" or buf[at + 4] != 2:
            raise ValueError("object header expected at %d" % at)
        flags = buf[at + 5]
        p = at + 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
        w = 1 << (flags & 3)
        size = int.from_bytes(buf[p:p + w], "little")
        p += w
        end = p + size
        if struct.unpack_from("<I", buf, end)[0] != lookup3(buf[at:end]):
            raise ValueError("object header checksum mismatch at %d" % at)
        links, attrs = {}, {}
        space = dtype = layout = None
        group = False
        while p + 4 <= end:
            mtype, msize, mflags = struct.unpack_from("<BHB", buf, p)
            p += 4 + (2 if flags & 0x04 else 0)
            body = buf[p:p + msize]
            p += msize
            if mtype == 2:
                group = True
            elif mtype == 6:
                lf = body[1]
                q = 2 + (1 if lf & 0x08 else 0) + (8 if lf & 0x04 else 0) + (1 if lf & 0x10 else 0)
                lw = 1 << (lf & 3)
                ln = int.from_bytes(body[q:q + lw], "little")
                q += lw
                links[body[q:q + ln].decode("ascii")] = struct.unpack_from("<Q", body, q + ln)[0]
            elif mtype == 1:
                space, _ = _parse_dataspace(body)
            elif mtype == 3:
                dtype, _ = _parse_datatype(body)
            elif mtype == 8:
                if body[0] != 3 or body[1] != 1:
                    raise ValueError("only contiguous layouts are read")
                layout = struct.unpack_from("<QQ", body, 2)
            elif mtype == 12:
                nsz, dsz, ssz = struct.unpack_from("<HHH", body, 2)
                q = 9
                name = body[q:q + nsz - 1].decode("ascii")
                q += nsz
                adt, _ = _parse_datatype(body[q:q + dsz])
                q += dsz
                ash, _ = _parse_dataspace(body[q:q + ssz])
                q += ssz
                attrs[name] = _decode(adt, ash, body[q:])
        if group:
            out = {k: node(a) for k, a in links.items()}
            if attrs:
                out["@attrs"] = attrs
            return out
        a, n = layout
        return _decode(dtype, space, buf[a:a + n])

    return node(root)
