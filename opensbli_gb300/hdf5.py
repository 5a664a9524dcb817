"""OPS-layout HDF5 output and restart files, written and read without libhdf5.

The generated code of the reference writes its results with OPS's ops_fetch_block_hdf5_file /
ops_fetch_dat_hdf5_file (core/io_hdf5.py:104-132, file opensbli_output.h5 or
opensbli_output_%06d.h5) and reads initial or restart data with ops_decl_dat_hdf5 from files laid out
by utilities/helperfunctions.py:80-127 (output_hdf5, set_hdf5_metadata): one group per block, named
after the block (opensbliblock00), with the attributes dims, ops_type = "ops_block" and index; one
dataset per array (rho_B0, ...), the array including its halos, with the attributes d_p, d_m, dim,
ops_type = "ops_dat", block_index, base, type = "double", block and size.

Neither machine this library targets has libhdf5 or h5py, so this module encodes the file format
itself, in its oldest and simplest form, following the HDF5 File Format Specification (version 0
superblock; version 1 object headers; groups as symbol tables: a version 1 B-tree group node over
symbol table nodes, and a local heap for the names; contiguous dataset storage; version 1 attribute, dataspace and
datatype messages; version 2 fill-value and version 3 layout messages).  Version 0 structures carry no
checksums.  `read_file` parses the same subset and checks every signature and version it meets.

Datasets are stored in C order with the shape [z][y][x] (2D: [y][x]), as OPS writes them.
"""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF      # the undefined address
HEAP_FREE_NULL = 1              # end of a local heap's free list, as libhdf5 encodes it
SIG = b"\x89HDF\r\n\x1a\n"
LEAF_K = 4                      # group leaf node K: a symbol table node holds 2K entries
INTERNAL_K = 16                 # group internal node K: a B-tree node holds 2K children
ENTRY_SIZE = 40                 # symbol table entry with 8-byte offsets and lengths
SNOD_SIZE = 8 + 2 * LEAF_K * ENTRY_SIZE
BTREE_SIZE = 24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8

# object header message types
MSG_DATASPACE, MSG_DATATYPE, MSG_FILL, MSG_LAYOUT, MSG_ATTRIBUTE, MSG_STAB = 0x1, 0x3, 0x5, 0x8, 0xC, 0x11


def _pad8(b):
    return b + b"\0" * (-len(b) % 8)


# ------------------------------------------------------------------------------------------ types
def _dtype_message(dt):
    """Datatype message body (version 1) for float64, int32 or fixed-length byte strings."""
    dt = np.dtype(dt)
    if dt == np.float64:
        # class 1 (floating point), little-endian, implied leading mantissa bit, sign at bit 63
        head = struct.pack("<B3BI", 0x11, 0x20, 63, 0, 8)
        return head + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
    if dt == np.int32:
        # class 0 (fixed point), little-endian, signed
        return struct.pack("<B3BI", 0x10, 0x08, 0, 0, 4) + struct.pack("<HH", 0, 32)
    if dt.kind == "S":
        # class 3 (string), null-padded ASCII
        return struct.pack("<B3BI", 0x13, 0x01, 0, 0, dt.itemsize)
    raise TypeError("unsupported HDF5 datatype %s" % dt)


def _parse_dtype(b):
    cls_ver, f0, f1, f2, size = struct.unpack_from("<B3BI", b, 0)
    cls, ver = cls_ver & 0x0F, cls_ver >> 4
    if ver != 1:
        raise ValueError("datatype message version %d" % ver)
    order = "<" if (f0 & 1) == 0 else ">"
    if cls == 1:
        return np.dtype(order + "f%d" % size)
    if cls == 0:
        return np.dtype(order + ("i" if f0 & 0x08 else "u") + "%d" % size)
    if cls == 3:
        return np.dtype("S%d" % size)
    raise ValueError("unsupported datatype class %d" % cls)


def _dataspace_message(shape):
    """Dataspace message body (version 1); shape () is a scalar."""
    return struct.pack("<BBBB4x", 1, len(shape), 0, 0) + b"".join(struct.pack("<Q", int(n)) for n in shape)


def _parse_dataspace(b):
    ver, rank, flags = struct.unpack_from("<BBB", b, 0)
    if ver != 1:
        raise ValueError("dataspace message version %d" % ver)
    return tuple(struct.unpack_from("<%dQ" % rank, b, 8)) if rank else ()


def _attribute_message(name, value):
    if isinstance(value, (str, bytes)):
        raw = value.encode("ascii") if isinstance(value, str) else value
        arr = np.array(raw, dtype="S%d" % max(len(raw), 1))
        shape = ()
    else:
        arr = np.asarray(value)
        if arr.dtype.kind in "iu":
            arr = arr.astype("<i4")
        elif arr.dtype.kind == "f":
            arr = arr.astype("<f8")
        shape = arr.shape
    dtm, dsm = _dtype_message(arr.dtype), _dataspace_message(shape)
    nm = name.encode("ascii") + b"\0"
    body = struct.pack("<BBHHH", 1, 0, len(nm), len(dtm), len(dsm))
    return body + _pad8(nm) + _pad8(dtm) + _pad8(dsm) + arr.tobytes()


def _parse_attribute(b):
    ver, _, nlen, tlen, slen = struct.unpack_from("<BBHHH", b, 0)
    if ver != 1:
        raise ValueError("attribute message version %d" % ver)
    p = 8
    name = b[p:p + nlen].split(b"\0", 1)[0].decode("ascii")
    p += nlen + (-nlen % 8)
    dt = _parse_dtype(b[p:p + tlen])
    p += tlen + (-tlen % 8)
    shape = _parse_dataspace(b[p:p + slen])
    p += slen + (-slen % 8)
    count = int(np.prod(shape)) if shape else 1
    arr = np.frombuffer(b[p:p + count * dt.itemsize], dtype=dt).reshape(shape)
    return name, (arr[()] if shape == () else arr.copy())


# ------------------------------------------------------------------------------------------ writer
class _File:
    """Append-only image of the file: structures are placed at 8-byte aligned addresses."""

    def __init__(self):
        self.buf = bytearray(96)  # the superblock, written last

    def alloc(self, nbytes):
        self.buf += b"\0" * (-len(self.buf) % 8)
        addr = len(self.buf)
        self.buf += b"\0" * nbytes
        return addr

    def put(self, addr, data):
        self.buf[addr:addr + len(data)] = data

    def object_header(self, messages):
        """Version 1 object header holding `messages` [(type, body, flags)]; returns its address."""
        chunk = b""
        for mtype, body, flags in messages:
            body = _pad8(body)
            chunk += struct.pack("<HHB3x", mtype, len(body), flags) + body
        head = struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(chunk))
        addr = self.alloc(len(head) + len(chunk))
        self.put(addr, head + chunk)
        return addr


def _entry(name_off, header_addr, cache=None):
    if cache is None:
        return struct.pack("<QQII16x", name_off, header_addr, 0, 0)
    return struct.pack("<QQIIQQ", name_off, header_addr, 1, 0, cache[0], cache[1])


def _write_group(f, children, attrs):
    """children: [(name, header_address, stab_cache or None)], names unique; returns (object header
    address, (B-tree address, heap address))."""
    if len(children) > 2 * LEAF_K * 2 * INTERNAL_K:
        raise ValueError("at most %d objects per group" % (2 * LEAF_K * 2 * INTERNAL_K))
    # local heap: "" at offset 0, then the names, each null-terminated and padded to 8 bytes
    data = b"\0" * 8
    offsets = {}
    for name, _, _ in children:
        offsets[name] = len(data)
        data += _pad8(name.encode("ascii") + b"\0")
    heap_data = f.alloc(len(data))
    f.put(heap_data, data)
    heap = f.alloc(32)
    f.put(heap, b"HEAP" + struct.pack("<B3xQQQ", 0, len(data), HEAP_FREE_NULL, heap_data))
    # symbol table nodes of up to 2K entries each, entries in name order
    ordered = sorted(children, key=lambda c: c[0].encode("ascii"))
    chunks = [ordered[i:i + 2 * LEAF_K] for i in range(0, len(ordered), 2 * LEAF_K)] or [[]]
    snods = []
    for ch in chunks:
        a = f.alloc(SNOD_SIZE)
        f.put(a, b"SNOD" + struct.pack("<BBH", 1, 0, len(ch)) + b"".join(_entry(offsets[n], h, c) for n, h, c in ch))
        snods.append(a)
    # one B-tree leaf (level 0) over them: keys are heap offsets of names; key 0 is "" (below every
    # name), key i+1 the last name of child i (at or above every name of child i, below child i+1's)
    btree = f.alloc(BTREE_SIZE)
    body = struct.pack("<Q", 0)
    for a, ch in zip(snods, chunks):
        body += struct.pack("<QQ", a, offsets[ch[-1][0]] if ch else 0)
    f.put(btree, b"TREE" + struct.pack("<BBHQQ", 0, 0, len(snods) if ordered else 0, UNDEF, UNDEF) + body)
    msgs = [(MSG_STAB, struct.pack("<QQ", btree, heap), 0)]
    msgs += [(MSG_ATTRIBUTE, _attribute_message(k, v), 0) for k, v in attrs.items()]
    return f.object_header(msgs), (btree, heap)


def _write_dataset(f, array, attrs):
    arr = np.ascontiguousarray(array, dtype="<f8")
    data = f.alloc(arr.nbytes)
    f.put(data, arr.tobytes())
    msgs = [(MSG_DATASPACE, _dataspace_message(arr.shape), 0),
            (MSG_DATATYPE, _dtype_message(np.float64), 1),
            # fill value message version 2: allocation time early, write time if set, no value
            (MSG_FILL, struct.pack("<BBBB", 2, 1, 2, 0), 0),
            (MSG_LAYOUT, struct.pack("<BBQQ", 3, 1, data, arr.nbytes), 0)]
    msgs += [(MSG_ATTRIBUTE, _attribute_message(k, v), 0) for k, v in attrs.items()]
    return f.object_header(msgs)


def write_file(path, blocks):
    """Write `blocks` = {group name: (group attributes, {dataset name: (float64 array, attributes)})}
    below the root group of a new file at `path`."""
    f = _File()
    entries = []
    for gname, (gattrs, dsets) in blocks.items():
        kids = [(dname, _write_dataset(f, arr, dattrs), None) for dname, (arr, dattrs) in dsets.items()]
        gaddr, gcache = _write_group(f, kids, gattrs)
        entries.append((gname, gaddr, gcache))
    raddr, rcache = _write_group(f, entries, {})
    f.buf += b"\0" * (-len(f.buf) % 8)
    eof = len(f.buf)
    sb = SIG + struct.pack("<8B", 0, 0, 0, 0, 0, 8, 8, 0) + struct.pack("<HHI", LEAF_K, INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF) + _entry(0, raddr, rcache)
    assert len(sb) == 96
    f.put(0, sb)
    with open(path, "wb") as fh:
        fh.write(bytes(f.buf))


# ------------------------------------------------------------------------------------------ reader
class _Reader:
    def __init__(self, b):
        self.b = b

    def messages(self, addr):
        ver, _, nmsg, _, size = struct.unpack_from("<BBHII", self.b, addr)
        if ver != 1:
            raise ValueError("object header version %d at %d" % (ver, addr))
        p, end, out = addr + 16, addr + 16 + size, []
        for _ in range(nmsg):
            mtype, msize, flags = struct.unpack_from("<HHB", self.b, p)
            out.append((mtype, bytes(self.b[p + 8:p + 8 + msize])))
            p += 8 + msize
            if p > end:
                raise ValueError("object header overrun at %d" % addr)
        return out

    def heap(self, addr):
        if self.b[addr:addr + 4] != b"HEAP" or self.b[addr + 4] != 0:
            raise ValueError("bad local heap at %d" % addr)
        size, free, data = struct.unpack_from("<QQQ", self.b, addr + 8)
        if free != HEAP_FREE_NULL and free >= size:
            raise ValueError("bad local heap free list at %d" % addr)
        return bytes(self.b[data:data + size])

    def group(self, btree, heap):
        names = self.heap(heap)
        out = []
        stack = [btree]
        while stack:
            a = stack.pop()
            if self.b[a:a + 4] != b"TREE":
                raise ValueError("bad B-tree node at %d" % a)
            ntype, level, used = struct.unpack_from("<BBH", self.b, a + 4)
            if ntype != 0:
                raise ValueError("B-tree node type %d in a group" % ntype)
            kids = [struct.unpack_from("<Q", self.b, a + 24 + 8 + 16 * i)[0] for i in range(used)]
            if level > 0:
                stack.extend(kids)
                continue
            for s in kids:
                if self.b[s:s + 4] != b"SNOD" or self.b[s + 4] != 1:
                    raise ValueError("bad symbol table node at %d" % s)
                (n,) = struct.unpack_from("<H", self.b, s + 6)
                for i in range(n):
                    off, hdr = struct.unpack_from("<QQ", self.b, s + 8 + ENTRY_SIZE * i)
                    out.append((names[off:names.index(b"\0", off)].decode("ascii"), hdr))
        return out

    def obj(self, addr):
        msgs = self.messages(addr)
        attrs = dict(_parse_attribute(b) for t, b in msgs if t == MSG_ATTRIBUTE)
        stab = [b for t, b in msgs if t == MSG_STAB]
        if stab:
            btree, heap = struct.unpack_from("<QQ", stab[0], 0)
            return {"attrs": attrs, "children": {n: self.obj(h) for n, h in self.group(btree, heap)}}
        shape = _parse_dataspace([b for t, b in msgs if t == MSG_DATASPACE][0])
        dt = _parse_dtype([b for t, b in msgs if t == MSG_DATATYPE][0])
        lay = [b for t, b in msgs if t == MSG_LAYOUT][0]
        ver, cls, daddr, dsize = struct.unpack_from("<BBQQ", lay, 0)
        if ver != 3 or cls != 1:
            raise ValueError("only contiguous layout (version 3) is read")
        arr = np.frombuffer(self.b[daddr:daddr + dsize], dtype=dt).reshape(shape).copy()
        return {"attrs": attrs, "data": arr}


def read_file(path):
    """Parse a file written by write_file (or any file within the same subset of the format):
    returns {"attrs": {...}, "children": {name: group or {"attrs", "data"}}} for the root group."""
    with open(path, "rb") as fh:
        b = fh.read()
    if b[:8] != SIG:
        raise ValueError("%s: not an HDF5 file" % path)
    if b[8] != 0 or b[13] != 8 or b[14] != 8:
        raise ValueError("%s: only superblock version 0 with 8-byte offsets and lengths is read" % path)
    (eof,) = struct.unpack_from("<Q", b, 40)
    if eof != len(b):
        raise ValueError("%s: end-of-file address %d, file size %d" % (path, eof, len(b)))
    (root,) = struct.unpack_from("<Q", b, 56 + 8)
    return _Reader(b).obj(root)


# ------------------------------------------------------------------------------------------ OPS layout
def ops_block_attrs(ndim, index=0):
    """Group attributes of an OPS block (helperfunctions.py:113-116)."""
    return {"dims": np.array([ndim], np.int32), "ops_type": b"ops_block", "index": np.array([index], np.int32)}


def ops_dat_attrs(npoints, halo, block_name, block_index=0):
    """Dataset attributes of an OPS dat (set_hdf5_metadata, helperfunctions.py:80-100): halo depth
    `halo` on every side of every axis, npoints interior points per axis (x first)."""
    nd = len(npoints)
    return {"d_p": np.full(nd, halo, np.int32), "d_m": np.full(nd, -halo, np.int32),
            "dim": np.array([1], np.int32), "ops_type": np.array(b"ops_dat", "S10"),
            "block_index": np.array([block_index], np.int32), "base": np.zeros(nd, np.int32),
            "type": np.array(b"double", "S15"), "block": np.array(block_name.encode("ascii"), "S25"),
            "size": np.array(npoints, np.int32)}


def write_ops_state(path, names, arrays, npoints, halo, block_name="opensbliblock00"):
    """One OPS block with one dat per conserved variable: arrays[v] is FP64 [z][y][x] (2D: [y][x])
    with `halo` points on every side; names are the dats' names (rho_B0, ...)."""
    nd = len(npoints)
    dsets = {}
    for name, arr in zip(names, arrays):
        arr = np.asarray(arr, dtype=np.float64)
        want = tuple(n + 2 * halo for n in reversed(npoints))
        if arr.shape != want:
            raise ValueError("%s: shape %s, expected %s" % (name, arr.shape, want))
        dsets[name] = (arr, ops_dat_attrs(npoints, halo, block_name))
    write_file(path, {block_name: (ops_block_attrs(nd), dsets)})


def read_ops_state(path, names, block_name="opensbliblock00"):
    """The dats `names` of one block: (list of FP64 arrays with their halos, halo depth, npoints)."""
    root = read_file(path)
    g = root["children"][block_name]
    out, halo, npts = [], None, None
    for name in names:
        d = g["children"][name]
        h = int(np.asarray(d["attrs"]["d_p"]).max())
        if int(-np.asarray(d["attrs"]["d_m"]).min()) != h or (halo is not None and h != halo):
            raise ValueError("%s: unequal halos" % name)
        halo, npts = h, tuple(int(v) for v in d["attrs"]["size"])
        out.append(d["data"])
    return out, halo, npts
