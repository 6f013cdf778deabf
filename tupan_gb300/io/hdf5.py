"""HDF5 files without h5py: the part of the format that tupan's snapshot and
worldline files use.

tupan/io/hdf5io.py:23-146 writes them through h5py with the HDF5 library's
default, earliest-compatible layout: a version-0 superblock, version-1 object
headers, groups stored as symbol tables (a version-1 B-tree of symbol nodes
whose names live in a local heap), datasets of one compound record per
particle, chunked with an unlimited maximum extent and compressed through the
shuffle and deflate filters, and a variable-length UTF-8 string attribute
"Class" on every group and dataset.  Neither h5py nor the HDF5 C library is
available to this package, so this module reads and writes that layout from
the published file-format specification (format version 0/1 structures).

`File(path, mode)` with mode "r" reads lazily.  Modes "w" (create or
truncate), "x"/"w-" (create, fail if present), "a" (read/write, create if
absent) and "r+" (read/write) load the group tree eagerly and write on
`close()`: new chunks, B-trees, heaps and object headers go to the end of the
file, object headers that already exist are patched in place (their
dataspace, layout and symbol-table messages keep their encoded sizes), and
the superblock is rewritten last.  Space held by replaced B-trees, heaps and
rewritten partial chunks is not reused.  A file left through an exception
(`with` block) or opened without a change is not written back: new chunks
may trail its end, unreferenced, and its structures are those it had.

Read as well (written by other producers of the same format version):
contiguous and compact storage, fixed-length strings, array datatypes and
compound members with dimensions, the Fletcher-32 filter (its checksum is
stripped, not verified), continuation blocks, user blocks.  Not read:
superblocks 2 and 3 and version-2 object headers (files made with
libver="latest"), link-message groups, shared and committed datatypes,
external and virtual storage; they raise NotImplementedError.
"""
import os
import struct
import zlib

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
HEAP_FREE_NULL = 1          # the end of a local heap's free list as stored on disk

MSG_NIL, MSG_DATASPACE, MSG_LINKINFO, MSG_DATATYPE = 0x0, 0x1, 0x2, 0x3
MSG_FILL_OLD, MSG_FILL, MSG_LINK, MSG_EXTERNAL = 0x4, 0x5, 0x6, 0x7
MSG_LAYOUT, MSG_PIPELINE, MSG_ATTRIBUTE = 0x8, 0xB, 0xC
MSG_CONTINUATION, MSG_SYMTAB = 0x10, 0x11

FILTER_DEFLATE, FILTER_SHUFFLE, FILTER_FLETCHER32 = 1, 2, 3

GROUP_LEAF_K, GROUP_INTERNAL_K, CHUNK_K = 4, 16, 32    # the library's defaults
GCOL_MIN = 4096                                        # smallest global heap collection
CHUNK_TARGET_BYTES = 8192                              # chunk size h5py picks for these datasets
DEFLATE_LEVEL = 4                                      # h5py's compression="gzip" default


_POOL = []
POOL_THREADS = max(1, min(8, (os.cpu_count() or 2) - 1))


def _pool():
    """Threads for chunk (de)compression, made on first use."""
    if not _POOL:
        from concurrent.futures import ThreadPoolExecutor
        _POOL.append(ThreadPoolExecutor(max_workers=POOL_THREADS, thread_name_prefix="hdf5-deflate"))
    return _POOL[0]


def _batches(n):
    """[lo, hi) ranges splitting n items into about four per pool thread."""
    nb = max(1, min(n, 4 * POOL_THREADS))
    return [(n * i // nb, n * (i + 1) // nb) for i in range(nb)]


def _pad8(n):
    return (n + 7) & ~7


def _cstr(buf, p):
    e = buf.index(b"\0", p)
    return buf[p:e].decode("utf-8", "surrogateescape")


class _VlenStr(object):
    """Marker for a variable-length string datatype (stored in a global heap)."""
    itemsize = 16

    def __init__(self, utf8):
        self.utf8 = utf8


# ---- datatypes --------------------------------------------------------------------------

def _decode_dtype(buf, p):
    """One datatype message at buf[p:] -> (numpy dtype or _VlenStr, end offset)."""
    cv = buf[p]
    cls, ver = cv & 0x0F, cv >> 4
    bf = buf[p + 1] | (buf[p + 2] << 8) | (buf[p + 3] << 16)
    size = struct.unpack_from("<I", buf, p + 4)[0]
    q = p + 8
    if cls == 0:                                    # fixed point
        order = ">" if bf & 1 else "<"
        dt = np.dtype("%s%s%d" % (order, "i" if bf & 0x8 else "u", size))
        q += 4
    elif cls == 1:                                  # floating point
        if bf & 0x40:
            raise NotImplementedError("VAX-order floating point")
        dt = np.dtype("%sf%d" % (">" if bf & 1 else "<", size))
        q += 12
    elif cls == 3:                                  # fixed-length string
        dt = np.dtype("S%d" % size)
    elif cls == 4:                                  # bit field
        dt = np.dtype("%su%d" % (">" if bf & 1 else "<", size))
        q += 4
    elif cls == 5:                                  # opaque
        n = buf.index(b"\0", q) - q
        q += _pad8(n + 1) if ver < 3 else n + 1
        dt = np.dtype("V%d" % size)
    elif cls == 6:                                  # compound
        names, formats, offsets = [], [], []
        for _ in range(bf & 0xFFFF):
            name = _cstr(buf, q)
            nb = len(name.encode("utf-8", "surrogateescape")) + 1
            q += _pad8(nb) if ver < 3 else nb
            if ver < 3:
                off = struct.unpack_from("<I", buf, q)[0]
                q += 4
            else:
                w = max(1, (size.bit_length() + 7) // 8)
                off = int.from_bytes(buf[q:q + w], "little")
                q += w
            dims = ()
            if ver == 1:
                nd = buf[q]
                dims = struct.unpack_from("<4I", buf, q + 12)[:nd]
                q += 28
            mdt, q = _decode_dtype(buf, q)
            if isinstance(mdt, _VlenStr):
                mdt = np.dtype("O")
            names.append(name)
            formats.append(np.dtype((mdt, dims)) if dims else mdt)
            offsets.append(off)
        dt = np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": size})
    elif cls == 9:                                  # variable length
        base, q = _decode_dtype(buf, q)
        if bf & 0xF == 1:
            return _VlenStr(((bf >> 8) & 0xF) == 1), q
        raise NotImplementedError("variable-length sequences")
    elif cls == 10:                                 # array
        nd = buf[q]
        q += 1 if ver >= 3 else 4
        dims = struct.unpack_from("<%dI" % nd, buf, q)
        q += 4 * nd
        if ver < 3:
            q += 4 * nd                             # permutation indices
        base, q = _decode_dtype(buf, q)
        dt = np.dtype((base, dims))
    else:
        raise NotImplementedError("datatype class %d" % cls)
    return dt, q


def _encode_dtype(dt):
    """numpy dtype (little-endian integers and IEEE floats, compounds of them,
    fixed-length byte strings) or _VlenStr -> datatype message bytes."""
    if isinstance(dt, _VlenStr):
        base = _encode_dtype(np.dtype("u1"))
        return bytes([0x19, 0x01, 0x01 if dt.utf8 else 0x00, 0x00]) + struct.pack("<I", 16) + base
    dt = np.dtype(dt)
    if dt.names is not None:
        body = b""
        for name in dt.names:
            fdt, off = dt.fields[name][:2]
            nb = name.encode("utf-8") + b"\0"
            body += nb + b"\0" * (_pad8(len(nb)) - len(nb))
            if fdt.subdtype is not None:
                base, shape = fdt.subdtype
                if len(shape) > 4:
                    raise NotImplementedError("compound member of rank > 4")
                dims = list(shape) + [0] * (4 - len(shape))
                body += struct.pack("<IB3xI4x4I", off, len(shape), 0, *dims) + _encode_dtype(base)
            else:
                body += struct.pack("<IB3xI4x4I", off, 0, 0, 0, 0, 0, 0) + _encode_dtype(fdt)
        n = len(dt.names)
        return bytes([0x16, n & 0xFF, (n >> 8) & 0xFF, 0]) + struct.pack("<I", dt.itemsize) + body
    if dt.byteorder == ">":
        raise NotImplementedError("big-endian datatypes are not written")
    if dt.kind in "iu":
        return bytes([0x10, 0x08 if dt.kind == "i" else 0x00, 0, 0]) + struct.pack("<IHH", dt.itemsize, 0, 8 * dt.itemsize)
    if dt.kind == "f":
        if dt.itemsize == 8:
            return bytes([0x11, 0x20, 63, 0]) + struct.pack("<IHHBBBBI", 8, 0, 64, 52, 11, 0, 52, 1023)
        if dt.itemsize == 4:
            return bytes([0x11, 0x20, 31, 0]) + struct.pack("<IHHBBBBI", 4, 0, 32, 23, 8, 0, 23, 127)
    if dt.kind == "S":
        return bytes([0x13, 0x00, 0, 0]) + struct.pack("<I", dt.itemsize)
    raise NotImplementedError("datatype %s" % dt)


# ---- the file ---------------------------------------------------------------------------

class _Node(object):
    def __init__(self, file, name, addr):
        self.file = file
        self.name = name
        self.addr = addr                # object header address, None until written
        self.attrs = {}
        self._new_attrs = []            # names to write with a new header

    def set_attr(self, key, value):
        """Attributes are stored as variable-length UTF-8 strings (what h5py
        writes for a Python str).  An existing object keeps its attributes;
        setting one again to the value it holds is allowed (the reference
        sets "Class" on every append)."""
        if not isinstance(value, str):
            raise TypeError("only string attributes are written")
        if key in self.attrs:
            if self.attrs[key] != value:
                raise NotImplementedError("changing attribute %r of an existing object" % key)
            return
        if self.addr is not None:
            raise NotImplementedError("adding attribute %r to an existing object" % key)
        self.file._check_writable()
        self.attrs[key] = value
        self._new_attrs.append(key)


class Group(_Node):
    def __init__(self, file, name, addr):
        _Node.__init__(self, file, name, addr)
        self._children = None           # name -> header address or node
        self._symtab_at = None          # file offset of the symbol-table message data
        self._dirty = addr is None

    # mapping interface
    def _entries(self):
        if self._children is None:
            self._children = self.file._read_group_entries(self)
        return self._children

    def keys(self):
        return sorted(self._entries(), key=lambda s: s.encode("utf-8"))

    def __contains__(self, key):
        return key in self._entries()

    def __iter__(self):
        return iter(self.keys())

    def __len__(self):
        return len(self._entries())

    def values(self):
        return [self[k] for k in self.keys()]

    def items(self):
        return [(k, self[k]) for k in self.keys()]

    def __getitem__(self, path):
        node = self
        for part in [p for p in path.split("/") if p]:
            ents = node._entries()
            if part not in ents:
                raise KeyError(path)
            child = ents[part]
            if not isinstance(child, _Node):
                child = node.file._load_node(node.name.rstrip("/") + "/" + part, child)
                ents[part] = child
            node = child
        return node

    def require_group(self, path):
        node = self
        for part in [p for p in path.split("/") if p]:
            if part in node:
                node = node[part]
                if not isinstance(node, Group):
                    raise TypeError("%r is not a group" % node.name)
            else:
                self.file._check_writable()
                child = Group(self.file, node.name.rstrip("/") + "/" + part, None)
                child._children = {}
                node._entries()[part] = child
                self.file._parents[id(child)] = node
                node._mark_dirty()
                node = child
        return node

    def _mark_dirty(self):
        g = self
        while g is not None:
            g._dirty = True
            g = self.file._parent_of(g)

    def append_rows(self, key, rows, level=DEFLATE_LEVEL):
        """Append the 1-D record array `rows` to dataset `key`, creating it
        chunked, of unlimited extent and shuffle+deflate compressed if absent
        (the dataset tupan/io/hdf5io.py:27-49 requires and resizes)."""
        rows = np.ascontiguousarray(rows)
        if rows.ndim != 1:
            raise ValueError("rows must be one-dimensional")
        if key in self:
            ds = self[key]
            if not isinstance(ds, Dataset):
                raise TypeError("%r is not a dataset" % ds.name)
        else:
            self.file._check_writable()
            ds = Dataset.create(self.file, self.name.rstrip("/") + "/" + key, rows.dtype, level)
            self._entries()[key] = ds
            self.file._parents[id(ds)] = self
            self._mark_dirty()
        ds.append(rows)
        return ds


class Dataset(_Node):
    def __init__(self, file, name, addr):
        _Node.__init__(self, file, name, addr)
        self.dtype = None
        self.shape = None
        self.maxshape = None
        self.layout = None              # ("compact", bytes) / ("contiguous", addr, size) / ("chunked", dims)
        self.filters = []               # (id, flags, client data)
        self._chunks = None             # chunk offset tuple -> (addr, stored bytes, filter mask)
        self._space_at = None           # file offset of the dataspace message data
        self._space_rank_max = None     # (version, rank, has maxdims) of that message
        self._layout_at = None          # file offset of the chunked layout's B-tree address
        self._dirty = False

    @classmethod
    def create(cls, file, name, dtype, level):
        ds = cls(file, name, None)
        ds.dtype = np.dtype(dtype)
        ds.shape = (0,)
        ds.maxshape = (None,)
        rows = 1
        while rows < 1024 and 2 * rows * ds.dtype.itemsize <= CHUNK_TARGET_BYTES:
            rows *= 2
        ds.layout = ("chunked", (rows,))
        ds.filters = [(FILTER_SHUFFLE, 1, (ds.dtype.itemsize,)), (FILTER_DEFLATE, 1, (int(level),))]
        ds._chunks = {}
        ds._dirty = True
        return ds

    def __len__(self):
        return self.shape[0] if self.shape else 1

    @property
    def chunks(self):
        return self.layout[1] if self.layout[0] == "chunked" else None

    def __getitem__(self, sel):
        return self.read()[sel]

    def read(self):
        return self.file._read_dataset(self)

    def append(self, rows):
        f = self.file
        f._check_writable()
        if self.layout[0] != "chunked" or len(self.shape) != 1 or self.maxshape[0] is not None:
            raise NotImplementedError("appending needs a 1-D chunked dataset of unlimited extent")
        if rows.dtype != self.dtype:
            if rows.dtype.names is None or self.dtype.names is None:
                rows = rows.astype(self.dtype)
            else:                                   # fields by name; the dataset's others are zero
                extra = set(rows.dtype.names) - set(self.dtype.names)
                if extra:
                    raise ValueError("fields %s are not in dataset %s" % (sorted(extra), self.name))
                conv = np.zeros(len(rows), dtype=self.dtype)
                for k in rows.dtype.names:
                    conv[k] = rows[k]
                rows = conv
        if self._chunks is None:
            self._chunks = f._read_chunk_index(self)
        c = self.layout[1][0]
        old, new = self.shape[0], self.shape[0] + len(rows)
        if new == old:
            return
        first = old // c
        buf = np.zeros((-(-new // c) - first) * c, dtype=self.dtype)
        if old % c:                                 # merge into the partial last chunk
            buf[:old % c] = f._read_chunk(self, (first * c,))[:old % c]
        buf[old % c:old % c + len(rows)] = rows
        f._write_chunks(self, first * c, buf)
        self.shape = (new,)
        self._dirty = True


class File(Group):
    """An HDF5 file; the root group."""

    def __init__(self, path, mode="r"):
        if mode not in ("r", "r+", "a", "w", "w-", "x"):
            raise ValueError("mode must be one of r, r+, a, w, w-, x")
        self.path = os.fspath(path)
        self.mode = mode
        self.file = self
        exists = os.path.exists(self.path)
        if mode in ("w-", "x") and exists:
            raise FileExistsError(self.path)
        create = mode in ("w", "w-", "x") or (mode == "a" and not exists)
        self._writable = mode != "r"
        self._fh = open(self.path, "w+b" if create else ("r+b" if self._writable else "rb"))
        self._parents = {}
        self._gheaps = {}
        self._closed = False
        self._changed = create          # nothing is written back unless something changed
        try:
            if create:
                Group.__init__(self, self, "/", None)
                self._children = {}
                self.sb_at, self.base = 0, 0
                self.leaf_k, self.internal_k, self.chunk_k = GROUP_LEAF_K, GROUP_INTERNAL_K, CHUNK_K
                self._sb_version = 0
                self._fh.write(b"\0" * 96)              # superblock, written on close
                self._eof = 96
            else:
                self._read_superblock()
                if self._writable:
                    self._load_tree(self)
        except BaseException:
            self._fh.close()
            raise

    # ---- context / lifetime
    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc, tb):
        if exc_type is None:
            self.close()
        else:                       # leave the file as it was: nothing linked, nothing patched
            self._changed = False
            self.close()

    def _check_writable(self):
        """Called before every change."""
        if not self._writable:
            raise ValueError("file %s is open read-only" % self.path)
        self._changed = True

    def close(self):
        if self._closed:
            return
        try:
            if self._writable and self._changed:
                self._flush()
        finally:
            self._fh.close()
            self._closed = True

    # ---- raw IO
    def _read(self, addr, n):
        self._fh.seek(self.base + addr)
        b = self._fh.read(n)
        if len(b) != n:
            raise ValueError("%s: truncated read at %d" % (self.path, addr))
        return b

    def _append(self, data, align=8):
        addr = _pad8(self._eof) if align else self._eof
        self._fh.seek(self.base + self._eof)
        self._fh.write(b"\0" * (addr - self._eof) + data)
        self._eof = addr + len(data)
        return addr

    def _patch(self, offset, data):
        self._fh.seek(self.base + offset)
        self._fh.write(data)

    # ---- superblock
    def _read_superblock(self):
        fh = self._fh
        fh.seek(0, 2)
        size = fh.tell()
        at = 0
        while True:
            fh.seek(at)
            if fh.read(8) == SIGNATURE:
                break
            at = 512 if at == 0 else 2 * at
            if at + 8 > size:
                raise ValueError("%s is not an HDF5 file" % self.path)
        fh.seek(at)
        sb = fh.read(128)
        ver = sb[8]
        if ver not in (0, 1):
            raise NotImplementedError("superblock version %d (a libver='latest' file)" % ver)
        if sb[13] != 8 or sb[14] != 8:
            raise NotImplementedError("offsets and lengths other than 8 bytes")
        self._sb_version = ver
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", sb, 16)
        p = 24
        self.chunk_k = CHUNK_K
        if ver == 1:
            self.chunk_k = struct.unpack_from("<H", sb, 24)[0]
            p = 28
        base, _free, eof, _drv = struct.unpack_from("<QQQQ", sb, p)
        self.sb_at, self.base = at, base
        _name, root_addr = struct.unpack_from("<QQ", sb, p + 32)
        Group.__init__(self, self, "/", root_addr)
        self._eof = max(eof, size) - base          # the stored end of file is absolute
        self._parse_node_header(self, root_addr)

    # ---- object headers
    def _messages(self, addr):
        """[(type, flags, absolute data offset, data)] of the object header at addr."""
        pre = self._read(addr, 16)
        if pre[:4] == b"OHDR":
            raise NotImplementedError("version-2 object headers (a libver='latest' file)")
        if pre[0] != 1:
            raise ValueError("object header version %d at %d" % (pre[0], addr))
        nmsg, _ref, size = struct.unpack_from("<HII", pre, 2)
        out, blocks = [], [(addr + 16, size)]
        while blocks:
            start, length = blocks.pop(0)
            buf = self._read(start, length)
            p = 0
            while p + 8 <= length:
                mtype, msize, mflags = struct.unpack_from("<HHB", buf, p)
                data = buf[p + 8:p + 8 + msize]
                if mtype == MSG_CONTINUATION:
                    blocks.append(struct.unpack_from("<QQ", data, 0))
                elif mtype != MSG_NIL:
                    if mflags & 0x2:
                        raise NotImplementedError("shared object header messages")
                    out.append((mtype, mflags, start + p + 8, data))
                p += 8 + msize
        return out

    def _parse_node_header(self, node, addr):
        for mtype, _fl, at, data in self._messages(addr):
            if mtype == MSG_SYMTAB:
                node._symtab_at = at
                node._btree, node._heap = struct.unpack_from("<QQ", data, 0)
            elif mtype in (MSG_LINK, MSG_LINKINFO):
                raise NotImplementedError("link-message groups (a libver='latest' file)")
            elif mtype == MSG_ATTRIBUTE:
                name, value = self._decode_attribute(data)
                node.attrs[name] = value

    def _load_node(self, name, addr):
        msgs = self._messages(addr)
        kinds = {m[0] for m in msgs}
        if MSG_SYMTAB in kinds:
            g = Group(self, name, addr)
            self._parse_node_header(g, addr)
            return g
        if MSG_LINK in kinds or MSG_LINKINFO in kinds:
            raise NotImplementedError("link-message groups (a libver='latest' file)")
        if MSG_LAYOUT not in kinds:
            raise NotImplementedError("object %s is neither a group nor a dataset" % name)
        ds = Dataset(self, name, addr)
        for mtype, _fl, at, data in msgs:
            if mtype == MSG_DATASPACE:
                ds.shape, ds.maxshape, ds._space_rank_max = self._decode_dataspace(data)
                ds._space_at = at
            elif mtype == MSG_DATATYPE:
                ds.dtype = _decode_dtype(data, 0)[0]
            elif mtype == MSG_LAYOUT:
                ds.layout, off = self._decode_layout(data)
                ds._layout_at = None if off is None else at + off
            elif mtype == MSG_PIPELINE:
                ds.filters = self._decode_pipeline(data)
            elif mtype == MSG_EXTERNAL:
                raise NotImplementedError("external storage")
            elif mtype == MSG_ATTRIBUTE:
                k, v = self._decode_attribute(data)
                ds.attrs[k] = v
        return ds

    def _load_tree(self, group):
        for k, v in list(group._entries().items()):
            child = group[k]
            self._parents[id(child)] = group
            if isinstance(child, Group):
                self._load_tree(child)

    def _parent_of(self, node):
        if node is self:
            return None
        p = self._parents.get(id(node))
        if p is None:                      # new nodes: find through the tree
            p = self._find_parent(self, node)
            self._parents[id(node)] = p
        return p

    def _find_parent(self, g, node):
        for v in (g._children or {}).values():
            if v is node:
                return g
            if isinstance(v, Group):
                r = self._find_parent(v, node)
                if r is not None:
                    return r
        return None

    # ---- messages
    @staticmethod
    def _decode_dataspace(data):
        ver, rank, flags = data[0], data[1], data[2]
        if ver == 1:
            p = 8
        elif ver == 2:
            p = 4
            if data[3] == 2:
                return None, None, (ver, 0, False)   # null dataspace
        else:
            raise NotImplementedError("dataspace version %d" % ver)
        dims = struct.unpack_from("<%dQ" % rank, data, p)
        maxd = None
        if flags & 1:
            m = struct.unpack_from("<%dQ" % rank, data, p + 8 * rank)
            maxd = tuple(None if x == UNDEF else x for x in m)
        return tuple(dims), maxd if maxd is not None else tuple(dims), (ver, rank, bool(flags & 1))

    @staticmethod
    def _decode_layout(data):
        ver = data[0]
        if ver in (1, 2):
            nd, cls = data[1], data[2]
            p = 8
            addr = None
            if cls != 0:
                addr = struct.unpack_from("<Q", data, p)[0]
                p += 8
            dims = struct.unpack_from("<%dI" % nd, data, p)
            p += 4 * nd
            if cls == 0:
                n = struct.unpack_from("<I", data, p)[0]
                return ("compact", data[p + 4:p + 4 + n]), None
            if cls == 1:
                return ("contiguous", addr, None), None
            return ("chunked", tuple(dims[:-1]), addr), 8
        if ver == 3:
            cls = data[1]
            if cls == 0:
                n = struct.unpack_from("<H", data, 2)[0]
                return ("compact", data[4:4 + n]), None
            if cls == 1:
                addr, size = struct.unpack_from("<QQ", data, 2)
                return ("contiguous", addr, size), None
            if cls == 2:
                nd = data[2]
                addr = struct.unpack_from("<Q", data, 3)[0]
                dims = struct.unpack_from("<%dI" % nd, data, 11)
                return ("chunked", tuple(dims[:-1]), addr), 3
            raise NotImplementedError("layout class %d" % cls)
        raise NotImplementedError("layout message version %d (a libver='latest' file)" % ver)

    @staticmethod
    def _decode_pipeline(data):
        ver, n = data[0], data[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = struct.unpack_from("<H", data, p)[0]
            p += 2
            nlen = 0
            if ver == 1 or fid >= 256:
                nlen = struct.unpack_from("<H", data, p)[0]
                p += 2
            flags, ncd = struct.unpack_from("<HH", data, p)
            p += 4
            p += _pad8(nlen) if ver == 1 else nlen
            cd = struct.unpack_from("<%dI" % ncd, data, p)
            p += 4 * ncd
            if ver == 1 and ncd % 2:
                p += 4
            out.append((fid, flags, cd))
        return out

    def _decode_attribute(self, data):
        ver = data[0]
        nname, ntype, nspace = struct.unpack_from("<HHH", data, 2)
        p = 8 if ver in (1, 2) else 9
        pad = _pad8 if ver == 1 else (lambda n: n)
        name = data[p:p + nname].split(b"\0")[0].decode("utf-8")
        p += pad(nname)
        dt = _decode_dtype(data, p)[0]
        p += pad(ntype)
        shape, _m, _v = self._decode_dataspace(data[p:p + nspace])
        p += pad(nspace)
        n = int(np.prod(shape)) if shape else 1
        if isinstance(dt, _VlenStr):
            vals = [self._vlen_str(data, p + 16 * i, dt.utf8) for i in range(n)]
            return name, vals[0] if not shape else np.array(vals, dtype=object).reshape(shape)
        arr = np.frombuffer(data, dtype=dt, count=n, offset=p)
        if not shape:
            v = arr[0]
            return name, v.decode("utf-8", "replace").rstrip("\0") if isinstance(v, bytes) else v
        return name, arr.reshape(shape).copy()

    def _vlen_str(self, buf, p, utf8):
        length, coll, idx = struct.unpack_from("<IQI", buf, p)
        if length == 0 or coll in (0, UNDEF):
            return ""
        raw = self._gheap_object(coll, idx)[:length]
        return raw.decode("utf-8" if utf8 else "ascii", "replace")

    def _gheap_object(self, coll, idx):
        objs = self._gheaps.get(coll)
        if objs is None:
            hdr = self._read(coll, 16)
            if hdr[:4] != b"GCOL":
                raise ValueError("no global heap collection at %d" % coll)
            size = struct.unpack_from("<Q", hdr, 8)[0]
            buf = self._read(coll, size)
            objs, p = {}, 16
            while p + 16 <= size:
                i, _r = struct.unpack_from("<HH", buf, p)
                n = struct.unpack_from("<Q", buf, p + 8)[0]
                if i == 0:
                    break
                objs[i] = buf[p + 16:p + 16 + n]
                p += 16 + _pad8(n)
            self._gheaps[coll] = objs
        return objs[idx]

    # ---- groups
    def _read_group_entries(self, g):
        if g.addr is None:
            return {}
        if not hasattr(g, "_btree"):
            self._parse_node_header(g, g.addr)
        if not hasattr(g, "_btree"):
            raise NotImplementedError("group %s has no symbol table" % g.name)
        heap = self._read(g._heap, 32)
        if heap[:4] != b"HEAP":
            raise ValueError("no local heap at %d" % g._heap)
        hsize, _free, haddr = struct.unpack_from("<QQQ", heap, 8)
        names = self._read(haddr, hsize)
        out = {}
        for snod in self._btree_children(g._btree, 0):
            hdr = self._read(snod, 8)
            if hdr[:4] != b"SNOD":
                raise ValueError("no symbol node at %d" % snod)
            n = struct.unpack_from("<H", hdr, 6)[0]
            ents = self._read(snod + 8, 40 * n)
            for i in range(n):
                noff, oaddr = struct.unpack_from("<QQ", ents, 40 * i)
                out[_cstr(names, noff)] = oaddr
        return out

    def _btree_children(self, addr, ntype, key_size=8):
        """Leaf children of the version-1 B-tree at addr, left to right, with
        the key before each for chunk trees: [(key bytes, child)] or [child]."""
        hdr = self._read(addr, 24)
        if hdr[:4] != b"TREE" or hdr[4] != ntype:
            raise ValueError("no type-%d B-tree node at %d" % (ntype, addr))
        level, n = hdr[5], struct.unpack_from("<H", hdr, 6)[0]
        body = self._read(addr + 24, n * (key_size + 8) + key_size)
        out = []
        for i in range(n):
            key = body[i * (key_size + 8):i * (key_size + 8) + key_size]
            child = struct.unpack_from("<Q", body, i * (key_size + 8) + key_size)[0]
            if level:
                out.extend(self._btree_children(child, ntype, key_size))
            else:
                out.append((key, child) if ntype == 1 else child)
        return out

    def _btree_walk(self, addr, ntype, ksz, levels):
        """The leaves' (key, child) of the B-tree at addr, left to right; every
        node visited is recorded in levels[level] (left to right) with its
        items, right key and sibling addresses."""
        hdr = self._read(addr, 24)
        if hdr[:4] != b"TREE" or hdr[4] != ntype:
            raise ValueError("no type-%d B-tree node at %d" % (ntype, addr))
        level, n = hdr[5], struct.unpack_from("<H", hdr, 6)[0]
        lsib, rsib = struct.unpack_from("<QQ", hdr, 8)
        body = self._read(addr + 24, n * (ksz + 8) + ksz)
        items = [(body[i * (ksz + 8):i * (ksz + 8) + ksz],
                  struct.unpack_from("<Q", body, i * (ksz + 8) + ksz)[0]) for i in range(n)]
        levels.setdefault(level, []).append({"addr": addr, "items": items, "right": body[n * (ksz + 8):],
                                             "lsib": lsib, "rsib": rsib})
        out = []
        for key, child in items:
            if level:
                out.extend(self._btree_walk(child, ntype, ksz, levels))
            else:
                out.append((key, child))
        return out

    # ---- dataset data
    def _read_chunk_index(self, ds):
        """offsets -> (address, stored bytes, filter mask) of every chunk; the
        index's nodes are kept (ds._tree) so that rewriting the index after
        an append writes only the nodes that change."""
        if ds.layout[0] != "chunked":
            return None
        addr = ds.layout[2] if len(ds.layout) > 2 else None
        if addr is None or addr == UNDEF:
            return {}
        rank = len(ds.layout[1])
        ksz = 8 + 8 * (rank + 1)
        out, levels = {}, {}
        for key, child in self._btree_walk(addr, 1, ksz, levels):
            nbytes, mask = struct.unpack_from("<II", key, 0)
            offs = struct.unpack_from("<%dQ" % rank, key, 8)
            out[offs] = (child, nbytes, mask)
        ds._tree = levels
        return out

    def _unfilter(self, ds, raw, mask):
        for i in range(len(ds.filters) - 1, -1, -1):
            fid, _fl, cd = ds.filters[i]
            if mask & (1 << i):
                continue
            if fid == FILTER_DEFLATE:
                raw = zlib.decompress(raw)
            elif fid == FILTER_SHUFFLE:
                s = cd[0] if cd else ds.dtype.itemsize
                n = len(raw) // s
                a = np.frombuffer(raw, np.uint8, count=n * s)
                raw = a.reshape(s, n).T.tobytes() + raw[n * s:]
            elif fid == FILTER_FLETCHER32:
                raw = raw[:-4]
            else:
                raise NotImplementedError("filter %d" % fid)
        return raw

    def _read_chunk(self, ds, offs):
        """The chunk at element offsets `offs` as a flat record array of the
        full chunk size (zeros where never written)."""
        dims = ds.layout[1]
        n = int(np.prod(dims))
        ent = ds._chunks.get(tuple(offs)) if ds._chunks is not None else None
        if ent is None:
            return np.zeros(n, dtype=ds.dtype)
        addr, nbytes, mask = ent
        raw = self._unfilter(ds, self._read(addr, nbytes), mask)
        return np.frombuffer(raw, dtype=ds.dtype, count=n).copy()

    def _read_dataset(self, ds):
        dt = ds.dtype
        if isinstance(dt, _VlenStr):
            raise NotImplementedError("datasets of variable-length strings")
        shape = ds.shape if ds.shape is not None else ()
        n = int(np.prod(shape)) if shape else 1
        kind = ds.layout[0]
        if kind == "compact":
            return np.frombuffer(ds.layout[1], dtype=dt, count=n).reshape(shape).copy()
        if kind == "contiguous":
            addr = ds.layout[1]
            if addr == UNDEF or n == 0:
                return np.zeros(shape, dtype=dt)
            return np.frombuffer(self._read(addr, n * dt.itemsize), dtype=dt).reshape(shape).copy()
        if ds._chunks is None:
            ds._chunks = self._read_chunk_index(ds)
        cdims = ds.layout[1]
        csize = int(np.prod(cdims))
        out = np.zeros(shape, dtype=dt)
        # the chunks inside the extent, read in file order, then unfiltered
        # on the thread pool (zlib releases the GIL) and placed
        items = sorted(((ent[0], offs, ent) for offs, ent in ds._chunks.items()
                        if all(o < s for o, s in zip(offs, shape))))
        raws = [self._read(addr, ent[1]) for addr, _offs, ent in items]

        def decode(lo_hi):
            return [self._unfilter(ds, raws[k], items[k][2][2]) for k in range(*lo_hi)]
        nch = len(items)
        if nch > 8:
            parts = _pool().map(decode, _batches(nch))
        else:
            parts = [decode((0, nch))]
        k = 0
        for part in parts:
            for raw in part:
                offs = items[k][1]
                k += 1
                chunk = np.frombuffer(raw, dtype=dt, count=csize).reshape(cdims)
                dst = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
                out[dst] = chunk[tuple(slice(0, d.stop - d.start) for d in dst)]
        return out

    def _write_chunks(self, ds, first, buf):
        """Write the whole chunks of record array `buf`, the first at element
        offset `first`: the shuffle of all chunks in one array operation,
        deflate of the chunks on a thread pool (zlib releases the GIL), the
        stored chunks appended in order."""
        c = ds.layout[1][0]
        nch = len(buf) // c
        s = ds.dtype.itemsize
        data = np.ascontiguousarray(buf).view(np.uint8).reshape(nch, c * s)
        level = None
        for fid, _fl, cd in ds.filters:
            if fid == FILTER_SHUFFLE:
                if cd[0] != s:
                    raise NotImplementedError("shuffle with an element size other than the record's")
                data = np.ascontiguousarray(data.reshape(nch, c, s).transpose(0, 2, 1)).reshape(nch, c * s)
            elif fid == FILTER_DEFLATE:
                level = cd[0] if cd else DEFLATE_LEVEL
            else:
                raise NotImplementedError("writing through filter %d" % fid)
        if level is None:
            rows = [data[k].tobytes() for k in range(nch)]
        else:
            def deflate(lo_hi):
                return [zlib.compress(data[k].tobytes(), level) for k in range(*lo_hi)]
            parts = _pool().map(deflate, _batches(nch)) if nch > 8 else [deflate((0, nch))]
            rows = [r for part in parts for r in part]
        for k, raw in enumerate(rows):
            addr = self._append(raw)
            ds._chunks[(first + k * c,)] = (addr, len(raw), 0)

    # ---- writing metadata
    def _flush(self):
        strings = []                                 # (node, key) of new vlen attributes
        self._collect_new_attrs(self, strings)
        gcol, ids = self._write_global_heap([self._node_attr(n, k) for n, k in strings])
        self._attr_ids = {(id(n), k): ids[i] for i, (n, k) in enumerate(strings)}
        self._gcol = gcol
        self._write_group(self)
        self._write_superblock()
        self._fh.flush()

    def _collect_new_attrs(self, g, out):
        for k in g._new_attrs:
            out.append((g, k))
        for v in (g._children or {}).values():
            if isinstance(v, _Node):
                if isinstance(v, Group):
                    self._collect_new_attrs(v, out)
                else:
                    out.extend((v, k) for k in v._new_attrs)

    @staticmethod
    def _node_attr(node, key):
        return node.attrs[key].encode("utf-8")

    def _write_global_heap(self, objs):
        if not objs:
            return None, []
        body = b""
        for i, o in enumerate(objs, start=1):
            body += struct.pack("<HHIQ", i, 0, 0, len(o)) + o + b"\0" * (_pad8(len(o)) - len(o))
        size = max(GCOL_MIN, 16 + len(body) + 16)
        free = size - 16 - len(body)
        data = b"GCOL" + bytes([1, 0, 0, 0]) + struct.pack("<Q", size) + body
        data += struct.pack("<HHIQ", 0, 0, 0, free) + b"\0" * (free - 16)
        return self._append(data), list(range(1, len(objs) + 1))

    def _attr_message(self, node, key):
        v = node.attrs[key]
        name = key.encode("utf-8") + b"\0"
        dt = _encode_dtype(_VlenStr(True))
        sp = bytes([1, 0, 0, 0, 0, 0, 0, 0])            # scalar dataspace
        ref = struct.pack("<IQI", len(v.encode("utf-8")), self._gcol, self._attr_ids[(id(node), key)])
        body = struct.pack("<BxHHH", 1, len(name), len(dt), len(sp))
        for part in (name, dt, sp):
            body += part + b"\0" * (_pad8(len(part)) - len(part))
        return MSG_ATTRIBUTE, 0, body + ref

    def _write_header(self, msgs):
        body = b""
        for mtype, flags, data in msgs:
            data = data + b"\0" * (_pad8(len(data)) - len(data))
            body += struct.pack("<HHB3x", mtype, len(data), flags) + data
        pre = struct.pack("<BxHII4x", 1, len(msgs), 1, len(body))
        return self._append(pre + body)

    def _write_dataset(self, ds):
        c = ds.layout[1][0]
        entries = sorted(ds._chunks.items())
        btree, ds._tree = self._write_chunk_btree(entries, c, ds.dtype.itemsize, getattr(ds, "_tree", None))
        if ds.addr is not None:
            ver, rank, hasmax = ds._space_rank_max
            self._patch(ds._space_at + (8 if ver == 1 else 4), struct.pack("<Q", ds.shape[0]))
            self._patch(ds._layout_at, struct.pack("<Q", btree))
            ds._dirty = False
            return
        space = struct.pack("<BBBx4xQQ", 1, 1, 1, ds.shape[0], UNDEF)
        fill = bytes([2, 3, 2, 0])                      # v2: incremental allocation, fill value undefined
        layout = struct.pack("<BBBQII", 3, 2, 2, btree, c, ds.dtype.itemsize)
        pl = struct.pack("<BB6x", 1, len(ds.filters))
        for fid, flags, cd in ds.filters:
            pl += struct.pack("<HHHH", fid, 0, flags, len(cd)) + struct.pack("<%dI" % len(cd), *cd)
            if len(cd) % 2:
                pl += b"\0" * 4
        msgs = [(MSG_DATASPACE, 0, space), (MSG_DATATYPE, 1, _encode_dtype(ds.dtype)), (MSG_FILL, 1, fill),
                (MSG_LAYOUT, 0, layout), (MSG_PIPELINE, 1, pl)]
        msgs += [self._attr_message(ds, k) for k in ds._new_attrs]
        ds.addr = self._write_header(msgs)
        ds._new_attrs = []
        ds._dirty = False

    def _write_chunk_btree(self, entries, c, itemsize, old=None):
        """Version-1 B-tree of the chunks (offset tuple -> (addr, bytes, mask)),
        built bottom-up with nodes of 2K entries allocated at full size; the key
        after the last chunk is its offset plus the chunk size.  A node of the
        previous index (`old`, per level) that holds the same entries is kept
        where it is, its right key and sibling links patched in place: an
        append rewrites only the nodes along the index's right edge.
        Returns (root address, the index's nodes per level)."""
        ksz = 24
        cap = 2 * self.chunk_k
        node_size = 24 + cap * 8 + (cap + 1) * ksz

        def key(nbytes, mask, off):
            return struct.pack("<IIQQ", nbytes, mask, off, 0)

        if not entries:
            return UNDEF, None                            # no chunk written yet: no index
        items = [(key(nb, m, offs[0]), addr) for offs, (addr, nb, m) in entries]
        last = key(0, 0, entries[-1][0][0] + c)
        levels, depth = {}, 0
        while True:
            nodes = self._btree_nodes(items, last, cap, node_size, 1, depth, ksz, (old or {}).get(depth))
            levels[depth] = nodes
            if len(nodes) == 1:
                return nodes[0]["addr"], levels
            items = [(nd["items"][0][0], nd["addr"]) for nd in nodes]
            depth += 1

    def _btree_nodes(self, items, last_key, cap, node_size, ntype, depth, ksz, old=None):
        """One level of B-tree nodes over `items` = [(key, child address)],
        2K to a node: a node of `old` with the same items is kept (its right
        key and sibling links patched if they changed), the others are
        written at the end of the file.  Returns the level's nodes."""
        groups = [items[i:i + cap] for i in range(0, len(items), cap)]
        keep = [old is not None and gi < len(old) and old[gi]["items"] == grp for gi, grp in enumerate(groups)]
        base, k, addrs = _pad8(self._eof), 0, []
        for gi in range(len(groups)):
            if keep[gi]:
                addrs.append(old[gi]["addr"])
            else:
                addrs.append(base + k * _pad8(node_size))
                k += 1
        out = []
        for gi, grp in enumerate(groups):
            right = groups[gi + 1][0][0] if gi + 1 < len(groups) else last_key
            lsib = addrs[gi - 1] if gi else UNDEF
            rsib = addrs[gi + 1] if gi + 1 < len(groups) else UNDEF
            if keep[gi]:
                o = old[gi]
                if o["right"] != right:
                    self._patch(o["addr"] + 24 + len(grp) * (ksz + 8), right)
                if o["lsib"] != lsib or o["rsib"] != rsib:
                    self._patch(o["addr"] + 8, struct.pack("<QQ", lsib, rsib))
            else:
                data = b"TREE" + bytes([ntype, depth]) + struct.pack("<HQQ", len(grp), lsib, rsib)
                for kb, child in grp:
                    data += kb + struct.pack("<Q", child)
                data += right
                data += b"\0" * (_pad8(node_size) - len(data))
                a = self._append(data)
                assert a == addrs[gi]
            out.append({"addr": addrs[gi], "items": grp, "right": right, "lsib": lsib, "rsib": rsib})
        return out

    def _write_group(self, g):
        """Write what changed below g, then g's symbol table (local heap, symbol
        nodes, B-tree) and, for a new group, its object header."""
        for k, v in (g._children or {}).items():
            if isinstance(v, Dataset) and (v._dirty or v.addr is None):
                self._write_dataset(v)
            elif isinstance(v, Group):
                self._write_group(v)
        if not g._dirty:
            return
        names = sorted(g._entries(), key=lambda s: s.encode("utf-8"))
        heap = b"\0" * 8
        offs = {}
        for nm in names:
            offs[nm] = len(heap)
            b = nm.encode("utf-8") + b"\0"
            heap += b + b"\0" * (_pad8(len(b)) - len(b))
        free = 16 + 8 * max(1, len(names))               # room the library can grow into
        heap_data = heap + struct.pack("<QQ", HEAP_FREE_NULL, free) + b"\0" * (free - 16)
        heap_addr = _pad8(self._eof)                     # header, then its data segment
        self._append(b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap_data), len(heap), heap_addr + 32)
                     + heap_data)
        per = 2 * self.leaf_k
        snod_size = 8 + per * 40
        items = []
        for i in range(0, len(names), per):
            chunk = names[i:i + per]
            data = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(chunk))
            for nm in chunk:
                data += self._symbol_entry(offs[nm], g._entries()[nm])
            a = self._append(data + b"\0" * (snod_size - len(data)))
            items.append((struct.pack("<Q", offs[chunk[-1]]), a))
        cap = 2 * self.internal_k
        node_size = 24 + cap * 8 + (cap + 1) * 8
        # key i: the largest name left of child i (key 0: the empty name at
        # heap offset 0); child i holds the names in (key i, key i+1]
        level = []
        prev = struct.pack("<Q", 0)
        for right, a in items:
            level.append((prev, a))
            prev = right
        if not level:                                    # an empty group: a root with no children
            data = b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", 0, UNDEF, UNDEF) + prev
            btree = self._append(data + b"\0" * (node_size - len(data)))
        else:
            depth = 0
            while True:
                nodes = self._btree_nodes(level, prev, cap, node_size, 0, depth, 8)
                if len(nodes) == 1:
                    btree = nodes[0]["addr"]
                    break
                level = [(nd["items"][0][0], nd["addr"]) for nd in nodes]
                depth += 1
        g._btree, g._heap = btree, heap_addr
        stab = struct.pack("<QQ", btree, heap_addr)
        if g.addr is not None:
            self._patch(g._symtab_at, stab)
        else:
            msgs = [(MSG_SYMTAB, 1, stab)] + [self._attr_message(g, k) for k in g._new_attrs]
            g.addr = self._write_header(msgs)
            g._new_attrs = []
            g._symtab_at = g.addr + 24                   # the first message's data
        g._dirty = False

    def _symbol_entry(self, name_off, node):
        if not isinstance(node, _Node):                  # unchanged, never loaded
            addr, cache = node, struct.pack("<II16x", 0, 0)
        elif isinstance(node, Group):
            addr, cache = node.addr, struct.pack("<IIQQ", 1, 0, node._btree, node._heap)
        else:
            addr, cache = node.addr, struct.pack("<II16x", 0, 0)
        return struct.pack("<QQ", name_off, addr) + cache

    def _write_superblock(self):
        root = struct.pack("<QQIIQQ", 0, self.addr, 1, 0, self._btree, self._heap)
        if self._sb_version == 0:
            sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", self.leaf_k, self.internal_k, 0)
        else:
            sb = SIGNATURE + bytes([1, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHIHH", self.leaf_k, self.internal_k, 0,
                                                                         self.chunk_k, 0)
        sb += struct.pack("<QQQQ", self.base, UNDEF, self.base + self._eof, UNDEF) + root
        self._fh.seek(self.sb_at)
        self._fh.write(sb)
