"""A small HDF5 writer and reader, written from the published HDF5 file
format specification (superblock version 0, version-1 object headers,
symbol-table groups with a version-1 B-tree, a local heap and symbol-table
nodes; contiguous datasets).  It covers what the final-state output needs
(output/mod.rs and main.rs:1289-1715 of the reference write it through
libhdf5 and the hdf5-writer crate):

- nested groups, and hard links that give one dataset a second name (the
  reference's aliases, e.g. `polarisation` for `polarization`);
- datasets of little-endian integers and IEEE floats, fixed-length UTF-8
  strings, enumerations over u8 (the boolean {false: 0, true: 1}, the
  laser's polarization and envelope), and arrays
  of four or three f64 per element (the reference's four- and
  three-vectors), either scalar or one-dimensional;
- fixed-length string attributes (`unit`, `desc`).

No libhdf5 exists in this environment, so `read` (the same subset) is the
checker the tests use.
"""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"
LEAF_K = 4        # symbol-table node holds 2 * LEAF_K entries
INTERNAL_K = 16   # group B-tree node holds 2 * INTERNAL_K children
ENTRY_SIZE = 40   # symbol-table entry with 8-byte offsets and lengths
SNOD_SIZE = 8 + 2 * LEAF_K * ENTRY_SIZE
TREE_SIZE = 24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8
HEAP_FREE_NULL = 1  # end of a local heap's free list

# message types
MSG_NIL, MSG_DATASPACE, MSG_DATATYPE, MSG_FILL, MSG_LAYOUT, MSG_ATTRIBUTE, MSG_STAB = 0, 1, 3, 5, 8, 12, 17


def _pad8(b):
    return b + b"\0" * (-len(b) % 8)


# ------------------------------------------------------------- datatypes ---
class Datatype:
    """An HDF5 datatype: `encode()` gives the datatype message body."""

    def __init__(self, cls, version, bits, size, props, numpy_dtype):
        self.cls, self.version, self.bits, self.size, self.props = cls, version, bits, size, props
        self.numpy_dtype = numpy_dtype

    def encode(self):
        head = bytes([(self.version << 4) | self.cls]) + struct.pack("<I", self.bits)[:3] + struct.pack("<I", self.size)
        return head + self.props


def fixed(nbytes, signed):
    bits = 0x08 if signed else 0x00  # little-endian, zero padding
    return Datatype(0, 1, bits, nbytes, struct.pack("<HH", 0, 8 * nbytes),
                    np.dtype(("<i%d" if signed else "<u%d") % nbytes))


def ieee(nbytes):
    if nbytes == 8:
        sign, eloc, esize, msize, bias = 63, 52, 11, 52, 1023
    else:
        sign, eloc, esize, msize, bias = 31, 23, 8, 23, 127
    bits = 0x20 | (sign << 8)  # little-endian, implied leading mantissa bit
    props = struct.pack("<HHBBBBI", 0, 8 * nbytes, eloc, esize, 0, msize, bias)
    return Datatype(1, 1, bits, nbytes, props, np.dtype("<f%d" % nbytes))


def string(nbytes):
    """Fixed-length, null-terminated UTF-8."""
    return Datatype(3, 1, 0x10, max(1, nbytes), b"", np.dtype("S%d" % max(1, nbytes)))


def enumeration(members):
    """An enumeration over u8: members = [(name, value), ...]."""
    base = fixed(1, False).encode()
    names = b"".join(_pad8(name.encode() + b"\0") for name, _ in members)
    values = bytes(v for _, v in members)
    return Datatype(8, 1, len(members), 1, base + names + values, np.dtype("u1"))


def boolean():
    """The enumeration {false: 0, true: 1} over u8 (what the reference
    writes for a Rust bool)."""
    return enumeration([("false", 0), ("true", 1)])


class Enum:
    """A scalar enumeration value to store: `members` [(name, value), ...]
    and the member `name`."""

    def __init__(self, members, name):
        self.members, self.value = members, dict(members)[name]


class Vector:
    """A single three- or four-vector to store as a scalar of the array
    datatype (the reference's ThreeVector, FourVector, StokesVector)."""

    def __init__(self, values):
        self.values = np.asarray(values, dtype="<f8").reshape(-1)


def array_f64(n):
    """An array of n f64 per element (datatype version 3)."""
    props = bytes([1]) + struct.pack("<I", n) + ieee(8).encode()
    return Datatype(10, 3, 0, 8 * n, props, np.dtype(("<f8", (n,))))


def _datatype_for(value):
    """(datatype, raw bytes, shape) for a value to store."""
    if isinstance(value, Vector):
        return array_f64(value.values.size), value.values.tobytes(), ()
    if isinstance(value, Enum):
        return enumeration(value.members), bytes([value.value]), ()
    if isinstance(value, (bool, np.bool_)):
        return boolean(), bytes([1 if value else 0]), ()
    if isinstance(value, str):
        b = value.encode("utf-8") + b"\0"
        return string(len(b)), b, ()
    if isinstance(value, (int, np.integer)) and not isinstance(value, (bool, np.bool_)):
        v = int(value)
        dt = fixed(8, False) if v >= 0 else fixed(8, True)
        return dt, np.array(v, dtype=dt.numpy_dtype).tobytes(), ()
    if isinstance(value, (float, np.floating)):
        return ieee(8), np.float64(value).tobytes(), ()
    a = np.asarray(value)
    if a.dtype == np.bool_:
        return boolean(), a.astype(np.uint8).tobytes(), a.shape
    if a.ndim == 2 and a.shape[1] in (3, 4) and a.dtype.kind == "f":
        return array_f64(a.shape[1]), np.ascontiguousarray(a, dtype="<f8").tobytes(), (a.shape[0],)
    if a.dtype.kind == "f":
        dt = ieee(a.dtype.itemsize)
    elif a.dtype.kind in "iu":
        dt = fixed(a.dtype.itemsize, a.dtype.kind == "i")
    else:
        raise TypeError("unsupported dataset type %s" % a.dtype)
    return dt, np.ascontiguousarray(a, dtype=dt.numpy_dtype).tobytes(), a.shape


def _dataspace(shape):
    """Dataspace message version 1 (rank 0 = scalar)."""
    b = bytes([1, len(shape), 0, 0]) + b"\0" * 4
    for d in shape:
        b += struct.pack("<Q", d)
    return b


# --------------------------------------------------------------- objects ---
class Dataset:
    def __init__(self, value):
        self.dtype, self.raw, self.shape = _datatype_for(value)
        self.attrs = {}
        self.links = 0
        self.addr = None

    def attr(self, name, text):
        self.attrs[name] = text
        return self


def _check_name(name):
    if not name or "/" in name or "\0" in name or name in (".", ".."):
        raise ValueError("invalid link name %r" % name)


class Group:
    def __init__(self):
        self.children = {}
        self.attrs = {}
        self.links = 0
        self.addr = None

    def group(self, name):
        _check_name(name)
        g = self.children.get(name)
        if g is None:
            g = self.children[name] = Group()
            g.links += 1
        if not isinstance(g, Group):
            raise ValueError("%r is a dataset" % name)
        return g

    def dataset(self, name, value, unit=None, desc=None, alias=None):
        _check_name(name)
        if alias is not None:
            _check_name(alias)
            if alias in self.children or alias == name:
                raise ValueError("%r exists" % alias)
        if name in self.children:
            raise ValueError("%r exists" % name)
        d = Dataset(value)
        if desc is not None:
            d.attr("desc", desc)
        if unit is not None:
            d.attr("unit", unit)
        self.children[name] = d
        d.links += 1
        if alias is not None:
            self.children[alias] = d  # a hard link: the same object header
            d.links += 1
        return d


def _message(mtype, body, flags=0):
    body = _pad8(body)
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _attribute(name, text):
    n = name.encode() + b"\0"
    b = text.encode("utf-8") + b"\0"
    dt = string(len(b)).encode()
    ds = _dataspace(())
    body = struct.pack("<BBHHH", 1, 0, len(n), len(dt), len(ds)) + _pad8(n) + _pad8(dt) + _pad8(ds) + b
    return _message(MSG_ATTRIBUTE, body)


def _object_header(messages, links):
    body = b"".join(messages)
    if not messages:
        body = _message(MSG_NIL, b"\0" * 8)
        messages = [body]
    return struct.pack("<BBHII4x", 1, 0, len(messages), links, len(body)) + body


class _Writer:
    def __init__(self):
        self.buf = bytearray(96)  # the superblock goes in at the end

    def alloc(self, data):
        addr = len(self.buf)
        self.buf += data
        self.buf += b"\0" * (-len(self.buf) % 8)
        return addr

    def reserve(self, n):
        addr = len(self.buf)
        self.buf += b"\0" * n
        return addr

    def put(self, addr, data):
        self.buf[addr:addr + len(data)] = data

    def dataset(self, d):
        if d.addr is not None:
            return
        data_addr = self.alloc(d.raw) if len(d.raw) else UNDEF
        msgs = [_message(MSG_DATASPACE, _dataspace(d.shape)), _message(MSG_DATATYPE, d.dtype.encode(), flags=1),
                _message(MSG_FILL, bytes([2, 2, 2, 0])),
                _message(MSG_LAYOUT, bytes([3, 1]) + struct.pack("<QQ", data_addr, len(d.raw)))]
        msgs += [_attribute(k, v) for k, v in d.attrs.items()]
        d.addr = self.alloc(_object_header(msgs, d.links))

    def group(self, g):
        """Writes g's members, then g's heap, symbol-table nodes, B-tree
        and object header.  Returns (header, B-tree, heap) addresses."""
        if g.addr is not None:
            return g.addr
        names = sorted(g.children, key=lambda s: s.encode())
        for name in names:
            c = g.children[name]
            if isinstance(c, Group):
                self.group(c)
            else:
                self.dataset(c)
        # local heap: "" at offset 0, then the names
        seg = bytearray(b"\0" * 8)
        off = {}
        for name in names:
            off[name] = len(seg)
            seg += _pad8(name.encode() + b"\0")
        seg_addr = self.alloc(bytes(seg))
        heap = b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(seg), HEAP_FREE_NULL, seg_addr)
        heap_addr = self.alloc(heap)
        # symbol-table nodes of at most 2 * LEAF_K entries (none for an empty
        # group, whose B-tree node then has no children)
        chunks = [names[i:i + 2 * LEAF_K] for i in range(0, len(names), 2 * LEAF_K)]
        if len(chunks) > 2 * INTERNAL_K:
            raise ValueError("group with more than %d members" % (4 * LEAF_K * INTERNAL_K))
        snods = []
        for chunk in chunks:
            b = bytearray(b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(chunk)))
            for name in chunk:
                b += self._entry(off[name], g.children[name])
            b += b"\0" * (SNOD_SIZE - len(b))
            snods.append(self.alloc(bytes(b)))
        tree = bytearray(b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", len(chunks), UNDEF, UNDEF))
        tree += struct.pack("<Q", 0)
        for chunk, addr in zip(chunks, snods):
            tree += struct.pack("<QQ", addr, off[chunk[-1]])
        tree += b"\0" * (TREE_SIZE - len(tree))
        tree_addr = self.alloc(bytes(tree))
        msgs = [_message(MSG_STAB, struct.pack("<QQ", tree_addr, heap_addr))]
        msgs += [_attribute(k, v) for k, v in g.attrs.items()]
        g.addr = (self.alloc(_object_header(msgs, max(1, g.links))), tree_addr, heap_addr)
        return g.addr

    def _entry(self, name_off, obj):
        if isinstance(obj, Group):
            hdr, tree, heap = obj.addr
            return struct.pack("<QQII", name_off, hdr, 1, 0) + struct.pack("<QQ", tree, heap)
        return struct.pack("<QQII", name_off, obj.addr, 0, 0) + b"\0" * 16


def write(path, root):
    """Writes the Group `root` as an HDF5 file."""
    w = _Writer()
    hdr, tree, heap = w.group(root)
    eof = len(w.buf)
    sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", LEAF_K, INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
    sb += struct.pack("<QQII", 0, hdr, 1, 0) + struct.pack("<QQ", tree, heap)
    assert len(sb) == 96
    w.put(0, sb)
    with open(path, "wb") as fh:
        fh.write(bytes(w.buf))


# ---------------------------------------------------------------- reader ---
class _Reader:
    def __init__(self, data):
        self.d = data
        if data[:8] != SIGNATURE:
            raise ValueError("not an HDF5 file")
        if data[8] != 0 or data[13] != 8 or data[14] != 8:
            raise ValueError("unsupported superblock")
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", data, 16)
        eof = struct.unpack_from("<Q", data, 40)[0]
        if eof != len(data):
            raise ValueError("end-of-file address %d, file size %d" % (eof, len(data)))
        self.root = struct.unpack_from("<Q", data, 64)[0]

    def header(self, addr):
        d = self.d
        version, _, nmsg, refs, size = struct.unpack_from("<BBHII", d, addr)
        if version != 1:
            raise ValueError("object header version %d" % version)
        p, end, msgs = addr + 16, addr + 16 + size, []
        for _ in range(nmsg):
            mtype, msize, flags = struct.unpack_from("<HHB", d, p)
            msgs.append((mtype, bytes(d[p + 8:p + 8 + msize])))
            p += 8 + msize
        if p != end:
            raise ValueError("object header size mismatch at %d" % addr)
        return msgs, refs

    def datatype(self, b, p=0):
        """(numpy dtype, kind, size, bytes used)."""
        cv = b[p]
        cls, version = cv & 15, cv >> 4
        bits = b[p + 1] | (b[p + 2] << 8) | (b[p + 3] << 16)
        size = struct.unpack_from("<I", b, p + 4)[0]
        q = p + 8
        if cls == 0:
            return np.dtype(("<i%d" if bits & 8 else "<u%d") % size), "int", size, 12
        if cls == 1:
            return np.dtype("<f%d" % size), "float", size, 20
        if cls == 3:
            return np.dtype("S%d" % size), "string", size, 8
        if cls == 8:
            nmem = bits & 0xFFFF
            _, _, bsize, used = self.datatype(b, q)
            q += used
            names = []
            for _ in range(nmem):
                e = b.index(b"\0", q)
                names.append(b[q:e].decode())
                q += (e - q + 1 + 7) // 8 * 8
            vals = list(b[q:q + nmem * bsize])
            q += nmem * bsize
            self.enum_names = dict(zip(vals, names))
            kind = "bool" if names == ["false", "true"] else "enum"
            return np.dtype("u%d" % bsize), kind, size, q - p
        if cls == 10 and version == 3:
            rank = b[q]
            dims = struct.unpack_from("<%dI" % rank, b, q + 1)
            q += 1 + 4 * rank
            base, _, _, used = self.datatype(b, q)
            return np.dtype((base, dims)), "array", size, q + used - p
        raise ValueError("unsupported datatype class %d version %d" % (cls, version))

    @staticmethod
    def dataspace(b, p=0):
        version, rank, flags = b[p], b[p + 1], b[p + 2]
        if version != 1:
            raise ValueError("dataspace version %d" % version)
        return tuple(struct.unpack_from("<%dQ" % rank, b, p + 8))

    def attributes(self, msgs):
        out = {}
        for mtype, b in msgs:
            if mtype != MSG_ATTRIBUTE:
                continue
            version, _, nlen, tlen, slen = struct.unpack_from("<BBHHH", b, 0)
            p = 8
            name = b[p:p + nlen - 1].decode()
            p += (nlen + 7) // 8 * 8
            dt, kind, size, _ = self.datatype(b, p)
            p += (tlen + 7) // 8 * 8
            p += (slen + 7) // 8 * 8
            raw = b[p:p + size]
            out[name] = raw.split(b"\0", 1)[0].decode("utf-8") if kind == "string" else raw
        return out

    def obj(self, addr):
        msgs, refs = self.header(addr)
        types = {t for t, _ in msgs}
        if MSG_STAB in types:
            tree, heap = struct.unpack_from("<QQ", dict(msgs)[MSG_STAB], 0)
            return {"kind": "group", "members": self.members(tree, heap), "attrs": self.attributes(msgs),
                    "refs": refs, "addr": addr}
        m = dict(msgs)
        shape = self.dataspace(m[MSG_DATASPACE])
        dt, kind, size, _ = self.datatype(m[MSG_DATATYPE])
        lay = m[MSG_LAYOUT]
        if lay[0] != 3 or lay[1] != 1:
            raise ValueError("layout version %d class %d" % (lay[0], lay[1]))
        daddr, dsize = struct.unpack_from("<QQ", lay, 2)
        n = int(np.prod(shape)) if shape else 1
        if dsize != n * size:
            raise ValueError("layout size %d for %d elements of %d bytes" % (dsize, n, size))
        raw = bytes(self.d[daddr:daddr + dsize]) if dsize else b""
        if kind == "string":
            value = raw.split(b"\0", 1)[0].decode("utf-8")
        else:
            a = np.frombuffer(raw, dtype=dt.base if kind == "array" else dt)
            if kind == "array":
                a = a.reshape((n,) + dt.shape)
            elif shape:
                a = a.reshape(shape)
            if kind == "bool":
                a = a.astype(bool)
            elif kind == "enum" and not shape:
                a = np.array(self.enum_names[int(a[0])], dtype=object)
            value = a if shape else a.reshape(()).item() if kind != "array" else a[0]
        return {"kind": "dataset", "value": value, "shape": shape, "type": kind, "attrs": self.attributes(msgs),
                "refs": refs, "addr": addr}

    def members(self, tree, heap):
        d = self.d
        if d[heap:heap + 4] != b"HEAP":
            raise ValueError("bad local heap")
        seg_size, free, seg = struct.unpack_from("<QQQ", d, heap + 8)
        if d[tree:tree + 4] != b"TREE" or d[tree + 4] != 0 or d[tree + 5] != 0:
            raise ValueError("bad group B-tree")
        nchild = struct.unpack_from("<H", d, tree + 6)[0]
        out, prev = {}, None
        for i in range(nchild):
            child = struct.unpack_from("<Q", d, tree + 24 + 8 + 16 * i)[0]
            if d[child:child + 4] != b"SNOD":
                raise ValueError("bad symbol-table node")
            nsym = struct.unpack_from("<H", d, child + 6)[0]
            for k in range(nsym):
                e = child + 8 + ENTRY_SIZE * k
                noff, oaddr = struct.unpack_from("<QQ", d, e)
                end = d.index(b"\0", seg + noff)
                name = bytes(d[seg + noff:end]).decode()
                if prev is not None and name.encode() <= prev.encode():
                    raise ValueError("symbols out of order: %r after %r" % (name, prev))
                prev = name
                out[name] = self.obj(oaddr)
        return out


def read(path):
    """The file's root group as nested dicts: a group is {"kind": "group",
    "members": {...}, "attrs": {...}}, a dataset {"kind": "dataset",
    "value": ..., "shape": ..., "type": ..., "attrs": {...}}."""
    with open(path, "rb") as fh:
        data = fh.read()
    r = _Reader(data)
    return r.obj(r.root)
