"""HDF5 files of the layout CyLag's mesh and field-set files use, without h5py.

The reference reads and writes its mesh (``TriangularMesh.from_hdf5`` /
``save_mesh_hdf5``, cylag/geom/triangular_mesh.pyx:204-290) and field-set
files (``EulerianFieldSet.from_hdf5`` / ``save_hdf5``,
cylag/core/eulerian_field_set.pyx:486-604) through h5py: one root group of
named datasets, each a numeric array, written with h5py's defaults.  h5py is
installed neither here nor on the GPU host, so this module reads and writes
that subset of the HDF5 file format (version 0 superblock, version 1 object
headers, symbol-table groups; contiguous, compact or unfiltered chunked
layouts; little- or big-endian integers and IEEE floats, fixed-length and
variable-length strings) from the format's published specification.

``read(path)`` returns ``{name: numpy array}`` for the root group's datasets
(variable-length strings as a list of ``bytes``); ``write(path, datasets)``
writes numeric arrays and lists of strings.  Anything outside the subset
(filters such as compression, external links, compound types) raises
``ValueError`` naming what was found.
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class _Reader:
    def __init__(self, data: bytes):
        self.d = data
        base = data.find(SIGNATURE)
        # the superblock may sit at 0, 512, 1024, ... (a user block before it)
        if base < 0 or base % 512:
            raise ValueError("not an HDF5 file (no superblock signature)")
        self.base = base
        ver = data[base + 8]
        if ver > 1:
            raise ValueError(f"HDF5 superblock version {ver}: only versions 0 and 1 are read")
        self.so = data[base + 13]   # size of offsets
        self.sl = data[base + 14]   # size of lengths
        if self.so != 8 or self.sl != 8:
            raise ValueError(f"HDF5 offsets/lengths of {self.so}/{self.sl} bytes: only 8 are read")
        p = base + 24 + (4 if ver == 1 else 0)
        self.base_addr = self.u(p, 8)
        # root group symbol table entry after base, free-space, EOF and
        # driver-info addresses
        self.root_entry = p + 32

    def u(self, p, n):
        return int.from_bytes(self.d[p:p + n], "little")

    def addr(self, a):
        return self.base_addr + a

    # ---- groups -----------------------------------------------------------
    def root_members(self):
        p = self.root_entry
        ohdr = self.u(p + 8, 8)
        cache = self.u(p + 16, 4)
        if cache == 1:
            btree, heap = self.u(p + 24, 8), self.u(p + 32, 8)
            return self._symbol_table(btree, heap)
        return self._group_from_header(ohdr)

    def _group_from_header(self, ohdr):
        msgs = self._messages(ohdr)
        for t, body in msgs:
            if t == 0x0011:
                return self._symbol_table(self._u(body, 0, 8), self._u(body, 8, 8))
        links = {}
        for t, body in msgs:
            if t == 0x0006:
                name, a = self._link(body)
                links[name] = a
        if links:
            return links
        raise ValueError("HDF5 group without a symbol table or compact links "
                         "(dense link storage is not read)")

    @staticmethod
    def _u(b, p, n):
        return int.from_bytes(b[p:p + n], "little")

    def _link(self, b):
        # link message (version 1): flags, [type], [creation order], [charset],
        # name length, name, hard link address
        if b[0] != 1:
            raise ValueError("HDF5 link message version %d" % b[0])
        flags = b[1]
        p = 2
        ltype = 0
        if flags & 0x8:
            ltype = b[p]
            p += 1
        if flags & 0x4:
            p += 8
        if flags & 0x10:
            p += 1
        nsize = 1 << (flags & 3)
        ln = self._u(b, p, nsize)
        p += nsize
        name = b[p:p + ln].decode("utf-8")
        p += ln
        if ltype != 0:
            raise ValueError(f"HDF5 link '{name}' is not a hard link")
        return name, self._u(b, p, 8)

    def _symbol_table(self, btree, heap):
        d = self.addr
        hp = d(heap)
        if self.d[hp:hp + 4] != b"HEAP":
            raise ValueError("HDF5 local heap signature missing")
        seg = d(self.u(hp + 24, 8))
        members = {}
        self._walk_group_btree(d(btree), seg, members)
        return members

    def _walk_group_btree(self, p, seg, members):
        if self.d[p:p + 4] != b"TREE":
            raise ValueError("HDF5 group B-tree signature missing")
        ntype, level, used = self.d[p + 4], self.d[p + 5], self.u(p + 6, 2)
        if ntype != 0:
            raise ValueError("HDF5 group B-tree of node type %d" % ntype)
        q = p + 8 + 16   # after the left and right sibling addresses
        for i in range(used):
            q += 8   # key i (heap offset)
            child = self.addr(self.u(q, 8))
            q += 8
            if level > 0:
                self._walk_group_btree(child, seg, members)
            else:
                self._snod(child, seg, members)

    def _snod(self, p, seg, members):
        if self.d[p:p + 4] != b"SNOD":
            raise ValueError("HDF5 symbol table node signature missing")
        n = self.u(p + 6, 2)
        q = p + 8
        for _ in range(n):
            off, ohdr = self.u(q, 8), self.u(q + 8, 8)
            end = self.d.index(b"\0", seg + off)
            members[self.d[seg + off:end].decode("utf-8")] = ohdr
            q += 40

    # ---- object headers ---------------------------------------------------
    def _messages(self, ohdr):
        p = self.addr(ohdr)
        if self.d[p:p + 4] == b"OHDR":
            return self._messages_v2(p)
        if self.d[p] != 1:
            raise ValueError("HDF5 object header version %d" % self.d[p])
        nmsg = self.u(p + 2, 2)
        size = self.u(p + 8, 4)
        blocks = [(p + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            q, n = blocks.pop(0)
            end = q + n
            while q + 8 <= end and len(out) < nmsg:
                t, sz = self.u(q, 2), self.u(q + 2, 2)
                body = self.d[q + 8:q + 8 + sz]
                out.append((t, body))
                if t == 0x0010:   # continuation
                    blocks.append((self.addr(self._u(body, 0, 8)), self._u(body, 8, 8)))
                q += 8 + sz
        return out

    def _messages_v2(self, p):
        flags = self.d[p + 5]
        q = p + 6
        if flags & 0x20:
            q += 16   # access, modification, change, birth times
        if flags & 0x10:
            q += 4    # attribute phase change values
        csize = 1 << (flags & 3)
        n = self.u(q, csize)
        q += csize
        blocks = [(q, n)]
        out = []
        track = bool(flags & 0x4)
        while blocks:
            q, n = blocks.pop(0)
            end = q + n
            while q + 4 <= end:
                t, sz = self.d[q], self.u(q + 1, 2)
                hdr = 4 + (2 if track else 0)
                body = self.d[q + hdr:q + hdr + sz]
                out.append((t, body))
                if t == 0x10:
                    a, ln = self._u(body, 0, 8), self._u(body, 8, 8)
                    blocks.append((self.addr(a) + 4, ln - 8))   # "OCHK" ... checksum
                q += hdr + sz
        return out

    # ---- datasets ---------------------------------------------------------
    def dataset(self, name, ohdr):
        shape = dtype = layout = None
        for t, body in self._messages(ohdr):
            if t == 0x0001:
                shape = self._dataspace(body)
            elif t == 0x0003:
                dtype = self._datatype(body)
            elif t == 0x0008:
                layout = body
            elif t == 0x000B:
                raise ValueError(f"HDF5 dataset '{name}' has a filter pipeline (compression); "
                                 "only unfiltered data are read")
        if shape is None or dtype is None or layout is None:
            raise ValueError(f"HDF5 object '{name}' is not a dataset")
        n = int(np.prod(shape, dtype=np.int64)) if shape else 1
        kind, arg = dtype
        esize = 16 if kind == "vlen" else arg.itemsize
        raw = self._raw(name, layout, n * esize, shape, esize)
        if kind == "vlen":
            return [self._vlen(raw[16 * i:16 * i + 16]) for i in range(n)]
        arr = np.frombuffer(raw, dtype=arg, count=n).copy()
        return arr.reshape(shape) if shape else arr.reshape(())

    def _dataspace(self, b):
        ver, ndim, flags = b[0], b[1], b[2]
        if ver == 1:
            p = 8
        elif ver == 2:
            p = 4
            if b[3] == 2:   # null dataspace
                return (0,)
        else:
            raise ValueError("HDF5 dataspace version %d" % ver)
        return tuple(self._u(b, p + 8 * i, 8) for i in range(ndim))

    def _datatype(self, b):
        cls, ver = b[0] & 0x0F, b[0] >> 4
        bits = b[1] | (b[2] << 8) | (b[3] << 16)
        size = self._u(b, 4, 4)
        order = ">" if bits & 1 else "<"
        if cls == 0:
            signed = bool(bits & 0x8)
            return "num", np.dtype(f"{order}{'i' if signed else 'u'}{size}")
        if cls == 1:
            if size not in (2, 4, 8):
                raise ValueError(f"HDF5 float of {size} bytes")
            return "num", np.dtype(f"{order}f{size}")
        if cls == 3:
            return "num", np.dtype(f"S{size}")
        if cls == 9:
            if (bits & 0xF) != 1:
                raise ValueError("HDF5 variable-length sequence (not a string)")
            return "vlen", None
        raise ValueError(f"HDF5 datatype class {cls} (version {ver}) is not read")

    def _raw(self, name, layout, nbytes, shape, esize):
        ver = layout[0]
        if ver == 3:
            cls = layout[1]
            if cls == 0:
                size = self._u(layout, 2, 2)
                return bytes(layout[4:4 + size])[:nbytes]
            if cls == 1:
                a = self._u(layout, 2, 8)
                if a == UNDEF:
                    return bytes(nbytes)   # never written: the fill value 0
                p = self.addr(a)
                return self.d[p:p + nbytes]
            if cls == 2:
                nd = layout[2]
                a = self._u(layout, 3, 8)
                cdims = [self._u(layout, 11 + 4 * i, 4) for i in range(nd)]
                return self._chunked(name, a, cdims[:-1], shape, esize)
            raise ValueError(f"HDF5 dataset '{name}': layout class {cls}")
        if ver in (1, 2):
            nd, cls = layout[1], layout[2]
            p = 8
            if cls in (1, 2):
                a = self._u(layout, p, 8)
                p += 8
            dims = [self._u(layout, p + 4 * i, 4) for i in range(nd)]
            p += 4 * nd
            if cls == 0:
                size = self._u(layout, p, 4)
                return bytes(layout[p + 4:p + 4 + size])[:nbytes]
            if cls == 1:
                q = self.addr(a)
                return self.d[q:q + nbytes]
            return self._chunked(name, a, dims[:-1], shape, esize)
        raise ValueError(f"HDF5 dataset '{name}': layout message version {ver}")

    def _chunked(self, name, btree, cdims, shape, esize):
        """Unfiltered chunks of a version 1 B-tree (node type 1) into one
        C-ordered buffer."""
        out = np.zeros(int(np.prod(shape, dtype=np.int64)) * esize, dtype=np.uint8)
        full = np.asarray(shape, dtype=np.int64)
        cd = np.asarray(cdims, dtype=np.int64)
        view = out.reshape(tuple(shape) + (esize,))
        nd = len(shape)

        def walk(p):
            if self.d[p:p + 4] != b"TREE" or self.d[p + 4] != 1:
                raise ValueError(f"HDF5 dataset '{name}': chunk B-tree signature missing")
            level, used = self.d[p + 5], self.u(p + 6, 2)
            ks = 8 + 8 * (nd + 1)   # chunk size, filter mask, offsets (+ element dim)
            q = p + 8 + 16
            for i in range(used):
                csize, mask = self.u(q, 4), self.u(q + 4, 4)
                offs = [self.u(q + 8 + 8 * j, 8) for j in range(nd)]
                child = self.addr(self.u(q + ks, 8))
                if level > 0:
                    walk(child)
                else:
                    if mask:
                        raise ValueError(f"HDF5 dataset '{name}': filtered chunk")
                    chunk = np.frombuffer(self.d[child:child + int(np.prod(cd)) * esize],
                                          dtype=np.uint8).reshape(tuple(cd) + (esize,))
                    o = np.asarray(offs, dtype=np.int64)
                    ext = np.minimum(cd, full - o)
                    dst = tuple(slice(int(a), int(a + e)) for a, e in zip(o, ext))
                    src = tuple(slice(0, int(e)) for e in ext)
                    view[dst] = chunk[src]
                q += ks + 8

        if btree != UNDEF:
            walk(self.addr(btree))
        return out.tobytes()

    def _vlen(self, e):
        n = self._u(e, 0, 4)
        coll, idx = self._u(e, 4, 8), self._u(e, 12, 4)
        if n == 0 or coll == 0:
            return b""
        p = self.addr(coll)
        if self.d[p:p + 4] != b"GCOL":
            raise ValueError("HDF5 global heap signature missing")
        size = self.u(p + 8, 8)
        q, end = p + 16, p + size
        while q + 16 <= end:
            oi, osz = self.u(q, 2), self.u(q + 8, 8)
            if oi == 0:
                break
            if oi == idx:
                return self.d[q + 16:q + 16 + osz][:n]
            q += 16 + ((osz + 7) // 8) * 8
        raise ValueError("HDF5 global heap object %d not found" % idx)


def read(path) -> dict:
    """The root group's datasets of an HDF5 file: {name: array} (variable-length
    strings as a list of bytes)."""
    r = _Reader(Path(path).read_bytes())
    return {name: r.dataset(name, ohdr) for name, ohdr in sorted(r.root_members().items())}


# ---------------------------------------------------------------------------
# writer: version 0 superblock, one symbol-table root group
# ---------------------------------------------------------------------------

def _pad8(b: bytes) -> bytes:
    return b + bytes(-len(b) % 8)


def _msg(mtype: int, body: bytes, flags: int = 0) -> bytes:
    body = _pad8(body)
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _object_header(messages: list) -> bytes:
    data = b"".join(messages)
    if len(data) < 32:   # the library's smallest object header chunk: a NIL message pads it
        messages = messages + [_msg(0x0000, bytes(32 - len(data) - 8))]
        data = b"".join(messages)
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(data)) + data


def _dtype_message(dt: np.dtype) -> bytes:
    order = 1 if dt.byteorder == ">" or (dt.byteorder == "=" and np.little_endian is False) else 0
    if dt.kind in "iu":
        bits = order | (0x8 if dt.kind == "i" else 0)
        return struct.pack("<B3BI", 0x10, bits, 0, 0, dt.itemsize) + struct.pack(
            "<HH", 0, 8 * dt.itemsize)
    if dt.kind == "f":
        if dt.itemsize == 8:
            eloc, esize, msize, bias = 52, 11, 52, 1023
        elif dt.itemsize == 4:
            eloc, esize, msize, bias = 23, 8, 23, 127
        else:
            raise ValueError(f"HDF5 writer: float of {dt.itemsize} bytes")
        sign = 8 * dt.itemsize - 1
        return struct.pack("<B3BI", 0x11, order | 0x20, sign, 0, dt.itemsize) + struct.pack(
            "<HHBBBBI", 0, 8 * dt.itemsize, eloc, esize, 0, msize, bias)
    if dt.kind == "S":
        return struct.pack("<B3BI", 0x13, 0, 0, 0, dt.itemsize)   # null-terminated ASCII
    raise ValueError(f"HDF5 writer: dtype {dt} is not written")


def _vlen_string_dtype_message() -> bytes:
    # variable-length string (UTF-8, null-terminated) of 1-byte characters
    base = struct.pack("<B3BI", 0x10, 0, 0, 0, 1) + struct.pack("<HH", 0, 8)
    return struct.pack("<B3BI", 0x19, 0x01, 0x01, 0, 16) + base


def _dataspace_message(shape) -> bytes:
    return struct.pack("<BBBB4x", 1, len(shape), 0, 0) + b"".join(
        struct.pack("<Q", int(n)) for n in shape)


def write(path, datasets: dict) -> None:
    """Write {name: array or list of str/bytes} as the root group's datasets.
    Numeric arrays keep their dtype (C order); a list of strings becomes a
    variable-length UTF-8 string dataset."""
    names = sorted(datasets)
    # local heap data: "" at offset 0, then each name null-terminated, 8-aligned
    heap = bytearray(8)
    name_off = {}
    for n in names:
        name_off[n] = len(heap)
        heap += _pad8(n.encode("utf-8") + b"\0")
    k_leaf = max(4, (len(names) + 1) // 2)   # one symbol node holds 2K entries
    sb_size = 96
    root_ohdr_size = len(_object_header([_msg(0x0011, bytes(16))]))
    heap_hdr = 32
    k_internal = 16
    # a group B-tree node is read at its full size: 2K children, 2K + 1 keys
    btree_size = 24 + 8 * (2 * k_internal) + 8 * (2 * k_internal + 1)
    snod_size = 8 + 40 * 2 * k_leaf
    pos = sb_size
    root_ohdr = pos
    pos += root_ohdr_size
    heap_addr = pos
    pos += heap_hdr
    heap_data_addr = pos
    pos += len(heap)
    btree_addr = pos
    pos += btree_size
    snod_addr = pos
    pos += snod_size
    blobs = []
    entries = []
    for n in names:
        v = datasets[n]
        if isinstance(v, (list, tuple)):
            strs = [s.encode("utf-8") if isinstance(s, str) else bytes(s) for s in v]
            # a global heap collection holding the strings
            objs = b"".join(struct.pack("<HH4xQ", i + 1, 1, len(s)) + _pad8(s)
                            for i, s in enumerate(strs))
            gsize = max(4096, 16 + len(objs) + 16)
            gcol_addr = pos
            free = gsize - 16 - len(objs)
            gcol = b"GCOL" + struct.pack("<B3xQ", 1, gsize) + objs + struct.pack(
                "<HH4xQ", 0, 0, free) + bytes(free - 16)
            pos += len(gcol)
            blobs.append(gcol)
            raw = b"".join(struct.pack("<IQI", len(s), gcol_addr, i + 1) for i, s in enumerate(strs))
            msgs = [_msg(0x0001, _dataspace_message((len(strs),))),
                    _msg(0x0003, _vlen_string_dtype_message(), flags=1)]
        else:
            a = np.ascontiguousarray(v)
            if a.dtype.byteorder == ">":
                a = a.astype(a.dtype.newbyteorder("<"))
            raw = a.tobytes()
            msgs = [_msg(0x0001, _dataspace_message(a.shape)),
                    _msg(0x0003, _dtype_message(a.dtype), flags=1)]
        data_addr = pos + len(_object_header(msgs + [_msg(0x0008, bytes(18))]))
        layout = struct.pack("<BBQQ", 3, 1, data_addr if raw else UNDEF, len(raw))
        oh = _object_header(msgs + [_msg(0x0008, layout)])
        entries.append((name_off[n], pos))
        blobs.append(oh + _pad8(raw))
        pos += len(oh) + len(_pad8(raw))
    eof = pos
    sb = SIGNATURE + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, k_leaf, k_internal, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
    sb += struct.pack("<QQII", 0, root_ohdr, 1, 0) + struct.pack("<QQ", btree_addr, heap_addr)
    root = _object_header([_msg(0x0011, struct.pack("<QQ", btree_addr, heap_addr))])
    # free-list head 1: the format's "no free block" offset
    hp = b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), 1, heap_data_addr)
    last = name_off[names[-1]] if names else 0
    bt = b"TREE" + struct.pack("<BBHQQ", 0, 0, 1 if names else 0, UNDEF, UNDEF)
    bt += struct.pack("<QQQ", 0, snod_addr, last)
    bt += bytes(btree_size - len(bt))
    snod = b"SNOD" + struct.pack("<BBH", 1, 0, len(names))
    for off, oh in entries:
        snod += struct.pack("<QQII16x", off, oh, 0, 0)
    snod += bytes(snod_size - len(snod))
    out = sb + root + hp + bytes(heap) + bt + snod + b"".join(blobs)
    assert len(out) == eof, (len(out), eof)
    Path(path).write_bytes(out)
