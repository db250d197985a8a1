"""Minimal HDF5 reader and writer without libhdf5 (the file I/O of reader.cpp
and Reader::writeData / writeSlab, reader.h:88-351).

Reader: superblock versions 0 and 1, old-style groups (symbol-table message,
version-1 group B-tree, local heap, symbol-table nodes), object headers
version 1 with continuation blocks, datasets with contiguous, compact or
chunked layout (version-1 chunk B-tree), filters deflate, shuffle and
fletcher32, fixed-point and IEEE floating-point element types, and attributes
of those types (for the `permute_order` attribute of reader.cpp:310-378).

Writer: superblock version 0, old-style groups (nested paths created on
demand), contiguous little-endian datasets of any numpy integer or float type
and optional attributes (fixed-length strings for `permute_order`) -- the
structures every HDF5 library version reads.

Format facts used here follow the published HDF5 File Format Specification
(version 2.0); nothing links to or reads libhdf5.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(RuntimeError):
    pass


# ---------------------------------------------------------------------------
# reading
# ---------------------------------------------------------------------------
class _Msg:
    __slots__ = ("type", "data")

    def __init__(self, t, data):
        self.type = t
        self.data = data


def _pad8(n):
    return (n + 7) & ~7


class H5File:
    """Read-only view of an HDF5 file held in memory."""

    def __init__(self, path_or_bytes):
        if isinstance(path_or_bytes, (bytes, bytearray, memoryview)):
            self.buf = bytes(path_or_bytes)
        else:
            with open(path_or_bytes, "rb") as f:
                self.buf = f.read()
        base = self._find_superblock()
        b = self.buf
        ver = b[base + 8]
        if ver not in (0, 1):
            raise H5Error(f"superblock version {ver} is not supported (only 0 and 1)")
        self.so, self.sl = b[base + 13], b[base + 14]
        if self.so != 8 or self.sl != 8:
            raise H5Error("only 8-byte offsets and lengths are supported")
        p = base + 24 + (4 if ver == 1 else 0)
        self.base = self._u(p, 8) if self._u(p, 8) != UNDEF else base
        p += 32  # base, free-space, end-of-file, driver-info addresses
        # root group symbol-table entry: name offset, object header address, ...
        self.root = self._u(p + 8, 8)

    # -- primitives --
    def _find_superblock(self):
        off = 0
        while off + 8 <= len(self.buf):
            if self.buf[off:off + 8] == SIGNATURE:
                return off
            off = 512 if off == 0 else off * 2
        raise H5Error("not an HDF5 file (no superblock signature)")

    def _u(self, off, n):
        return int.from_bytes(self.buf[off:off + n], "little")

    def _addr(self, a):
        return a + self.base

    # -- object headers --
    def _messages(self, addr):
        b = self.buf
        a = self._addr(addr)
        if b[a] != 1:
            raise H5Error(f"object header version {b[a]} at {addr:#x} is not supported (only version 1)")
        nmsg = self._u(a + 2, 2)
        size = self._u(a + 8, 4)
        blocks = [(a + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p, end = start, start + length
            while p + 8 <= end and len(out) < nmsg:
                t, sz = self._u(p, 2), self._u(p + 2, 2)
                data = b[p + 8:p + 8 + sz]
                p += 8 + sz
                if t == 0x10:  # continuation
                    blocks.append((self._addr(int.from_bytes(data[0:8], "little")),
                                   int.from_bytes(data[8:16], "little")))
                out.append(_Msg(t, data))
        return out

    # -- groups --
    def _heap_data(self, heap_addr):
        a = self._addr(heap_addr)
        if self.buf[a:a + 4] != b"HEAP":
            raise H5Error("bad local heap signature")
        return self._addr(self._u(a + 24, 8))

    def _heap_str(self, data_addr, off):
        s = self.buf[data_addr + off:]
        return s[:s.index(b"\0")].decode()

    def _group_entries(self, btree_addr, heap_addr):
        data = self._heap_data(heap_addr)
        entries = {}

        def walk(node):
            a = self._addr(node)
            if self.buf[a:a + 4] != b"TREE":
                raise H5Error("bad group B-tree signature")
            level, used = self.buf[a + 5], self._u(a + 6, 2)
            p = a + 24  # after signature, type, level, entries, siblings
            children = []
            for i in range(used):
                p += 8  # key (heap offset)
                children.append(self._u(p, 8))
                p += 8
            for c in children:
                if level > 0:
                    walk(c)
                else:
                    s = self._addr(c)
                    if self.buf[s:s + 4] != b"SNOD":
                        raise H5Error("bad symbol-table node signature")
                    n = self._u(s + 6, 2)
                    q = s + 8
                    for _ in range(n):
                        name = self._heap_str(data, self._u(q, 8))
                        entries[name] = self._u(q + 8, 8)
                        q += 40

        walk(btree_addr)
        return entries

    @staticmethod
    def _link(d):
        """Link message (type 0x06), hard links only: (name, object header address)."""
        flags = d[1]
        p = 2
        ltype = 0
        if flags & 0x08:
            ltype = d[p]
            p += 1
        if flags & 0x04:
            p += 8  # creation order
        if flags & 0x10:
            p += 1  # name character set
        nsz = 1 << (flags & 0x03)
        nlen = int.from_bytes(d[p:p + nsz], "little")
        p += nsz
        name = d[p:p + nlen].decode()
        p += nlen
        if ltype != 0:
            return name, None  # soft / external links are not followed
        return name, int.from_bytes(d[p:p + 8], "little")

    def _children(self, obj_addr):
        """Members of a group: old-style (symbol table) or compact new-style (link messages)."""
        links, is_group, dense = {}, False, False
        for m in self._messages(obj_addr):
            if m.type == 0x11:
                bt, hp = struct.unpack_from("<QQ", m.data, 0)
                return self._group_entries(bt, hp)
            if m.type == 0x02:
                is_group = True
                flags = m.data[1]
                fheap = struct.unpack_from("<Q", m.data, 2 + (8 if flags & 1 else 0))[0]
                dense = fheap != UNDEF
            elif m.type == 0x06:
                is_group = True
                name, addr = self._link(m.data)
                if addr is not None:
                    links[name] = addr
        if dense and not links:
            raise H5Error("groups with dense link storage (fractal heap) are not supported")
        return links if is_group else None

    def _resolve(self, path):
        addr = self.root
        for part in [p for p in path.split("/") if p]:
            ch = self._children(addr)
            if ch is None or part not in ch:
                raise KeyError(f"{path}: '{part}' not found")
            addr = ch[part]
        return addr

    def keys(self, path="/"):
        ch = self._children(self._resolve(path))
        return sorted(ch) if ch is not None else []

    def is_group(self, path):
        return self._children(self._resolve(path)) is not None

    # -- datasets --
    @staticmethod
    def _dtype(d):
        cls, ver = d[0] & 0x0F, d[0] >> 4
        if cls == 9 and (d[1] & 0x0F) == 1:
            return "vlen_str"  # variable-length string: (length, global heap address, index) per element
        bits = d[1] | (d[2] << 8) | (d[3] << 16)
        size = int.from_bytes(d[4:8], "little")
        order = ">" if bits & 1 else "<"
        if cls == 0:
            signed = bool(bits & 0x08)
            return np.dtype(f"{order}{'i' if signed else 'u'}{size}")
        if cls == 1:
            if size not in (2, 4, 8):
                raise H5Error(f"floating-point size {size} not supported")
            return np.dtype(f"{order}f{size}")
        if cls == 3:
            return np.dtype(f"S{size}")
        raise H5Error(f"datatype class {cls} (version {ver}) not supported")

    @staticmethod
    def _dataspace(d):
        ver, nd, flags = d[0], d[1], d[2]
        p = 8 if ver == 1 else 4
        if ver == 2 and d[3] == 0:
            return ()  # scalar
        dims = struct.unpack_from(f"<{nd}Q", d, p)
        return tuple(int(x) for x in dims)

    def _global_heap_object(self, addr, index):
        """Object `index` of the global heap collection at `addr` (GCOL)."""
        a = self._addr(addr)
        if self.buf[a:a + 4] != b"GCOL":
            raise H5Error("bad global heap collection signature")
        size = self._u(a + 8, 8)
        p, end = a + 16, a + size
        while p + 16 <= end:
            idx, osz = self._u(p, 2), self._u(p + 8, 8)
            if idx == 0:
                break
            if idx == index:
                return self.buf[p + 16:p + 16 + osz]
            p += 16 + _pad8(osz)
        raise H5Error(f"global heap object {index} not found")

    def _read_attr(self, d):
        ver = d[0]
        nlen, tlen, slen = struct.unpack_from("<HHH", d, 2)
        if ver == 1:
            p = 8
            name = d[p:p + nlen].split(b"\0")[0].decode()
            p += _pad8(nlen)
            dt = self._dtype(d[p:p + tlen])
            p += _pad8(tlen)
            shape = self._dataspace(d[p:p + slen])
            p += _pad8(slen)
        else:
            p = 8 if ver == 2 else 9
            name = d[p:p + nlen].split(b"\0")[0].decode()
            p += nlen
            dt = self._dtype(d[p:p + tlen])
            p += tlen
            shape = self._dataspace(d[p:p + slen])
            p += slen
        count = int(np.prod(shape)) if shape else 1
        if isinstance(dt, str):  # variable-length strings
            vals = []
            for k in range(count):
                q = p + 16 * k
                ln = int.from_bytes(d[q:q + 4], "little")
                addr = int.from_bytes(d[q + 4:q + 12], "little")
                idx = int.from_bytes(d[q + 12:q + 16], "little")
                vals.append(self._global_heap_object(addr, idx)[:ln].decode("utf-8") if ln else "")
            return name, vals[0] if not shape else vals
        arr = np.frombuffer(d, dtype=dt, count=count, offset=p).copy()
        return name, arr.reshape(shape) if shape else arr[0]

    def attrs(self, path):
        out = {}
        for m in self._messages(self._resolve(path)):
            if m.type == 0x0C:
                k, v = self._read_attr(m.data)
                out[k] = v
        return out

    def read(self, path):
        """Dataset `path` as a numpy array in its stored (C) order."""
        msgs = self._messages(self._resolve(path))
        shape = dt = layout = None
        filters = []
        for m in msgs:
            if m.type == 0x01:
                shape = self._dataspace(m.data)
            elif m.type == 0x03:
                dt = self._dtype(m.data)
            elif m.type == 0x08:
                layout = m.data
            elif m.type == 0x0B:
                filters = self._filters(m.data)
        if shape is None or dt is None or layout is None:
            raise H5Error(f"{path} is not a dataset")
        count = int(np.prod(shape)) if shape else 1
        ver = layout[0]
        if ver != 3:
            raise H5Error(f"data layout version {ver} not supported (only 3)")
        cls = layout[1]
        if cls == 0:  # compact
            sz = struct.unpack_from("<H", layout, 2)[0]
            raw = layout[4:4 + sz]
            return np.frombuffer(raw, dtype=dt, count=count).reshape(shape).copy()
        if cls == 1:  # contiguous
            addr, sz = struct.unpack_from("<QQ", layout, 2)
            if addr == UNDEF:
                return np.zeros(shape, dtype=dt)
            a = self._addr(addr)
            return np.frombuffer(self.buf, dtype=dt, count=count, offset=a).reshape(shape).copy()
        if cls == 2:  # chunked
            nd = layout[2]
            bt = struct.unpack_from("<Q", layout, 3)[0]
            cdims = struct.unpack_from(f"<{nd}I", layout, 11)
            return self._read_chunked(bt, shape, dt, cdims[:-1], filters)
        raise H5Error(f"layout class {cls} not supported")

    @staticmethod
    def _filters(d):
        ver, n = d[0], d[1]
        out = []
        p = 8 if ver == 1 else 2
        for _ in range(n):
            fid = struct.unpack_from("<H", d, p)[0]
            if ver == 1 or fid >= 256:
                nlen = struct.unpack_from("<H", d, p + 2)[0]
                flags, nval = struct.unpack_from("<HH", d, p + 4)
                p += 8
                p += _pad8(nlen) if ver == 1 else nlen
            else:
                flags, nval = struct.unpack_from("<HH", d, p + 2)
                p += 6
            vals = struct.unpack_from(f"<{nval}I", d, p)
            p += 4 * nval
            if ver == 1 and nval % 2:
                p += 4
            out.append((fid, vals))
        return out

    def _read_chunked(self, bt, shape, dt, cdims, filters):
        out = np.zeros(shape, dtype=dt)
        nd = len(shape)
        esz = dt.itemsize

        def walk(node):
            a = self._addr(node)
            if self.buf[a:a + 4] != b"TREE" or self.buf[a + 4] != 1:
                raise H5Error("bad chunk B-tree node")
            level, used = self.buf[a + 5], self._u(a + 6, 2)
            p = a + 24
            ksz = 8 + 8 * (nd + 1)
            for _ in range(used):
                csize, fmask = struct.unpack_from("<II", self.buf, p)
                offs = struct.unpack_from(f"<{nd}Q", self.buf, p + 8)
                child = self._u(p + ksz, 8)
                p += ksz + 8
                if level > 0:
                    walk(child)
                    continue
                raw = self.buf[self._addr(child):self._addr(child) + csize]
                for i, (fid, vals) in reversed(list(enumerate(filters))):
                    if fmask & (1 << i):
                        continue
                    if fid == 1:
                        raw = zlib.decompress(raw)
                    elif fid == 2:
                        n = len(raw) // esz
                        raw = np.frombuffer(raw, np.uint8).reshape(esz, n).T.tobytes()
                    elif fid == 3:
                        raw = raw[:-4]
                    else:
                        raise H5Error(f"filter {fid} not supported")
                chunk = np.frombuffer(raw, dtype=dt, count=int(np.prod(cdims))).reshape(cdims)
                sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
                out[sl] = chunk[tuple(slice(0, s.stop - s.start) for s in sl)]

        if bt != UNDEF:
            walk(bt)
        return out


def read_microstructure(path, dataset):
    """Reader::ReadMS (reader.cpp:227-411): the phase-id array in [x][y][z]
    order.  The dataset is taken as ZYX (reader.h:54) unless a `permute_order`
    attribute starts with something other than 'z' (reader.cpp:262-273); a ZYX
    dataset is transposed to XYZ (reader.cpp:383-396)."""
    f = H5File(path)
    ms = f.read(dataset)
    if ms.ndim != 3:
        raise H5Error(f"{dataset}: microstructure must be 3-D, got shape {ms.shape}")
    attrs = f.attrs(dataset)
    is_zyx = True  # reader.h:54
    if "permute_order" in attrs:
        order = attrs["permute_order"]
        order = order.decode() if isinstance(order, (bytes, np.bytes_)) else str(order)
        is_zyx = order[:1] in ("z", "Z")  # reader.cpp:268
    if is_zyx:
        ms = np.ascontiguousarray(np.transpose(ms, (2, 1, 0)))
    return ms


# ---------------------------------------------------------------------------
# writing
# ---------------------------------------------------------------------------
class _Node:
    def __init__(self):
        self.children = {}  # name -> _Node | (ndarray, attrs)
        self.attrs = {}


def _dtype_msg(dt):
    dt = np.dtype(dt).newbyteorder("<") if np.dtype(dt).byteorder == ">" else np.dtype(dt)
    size = dt.itemsize
    if dt.kind in "iu":
        bits = 0x08 if dt.kind == "i" else 0
        return struct.pack("<BBBBI", 0x10 | 0, bits, 0, 0, size) + struct.pack("<HH", 0, 8 * size)
    if dt.kind == "f":
        # IEEE little endian: sign location, exponent/mantissa fields
        if size == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            return struct.pack("<BBBBI", 0x11, 0x20, 63, 0, 8) + props
        if size == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            return struct.pack("<BBBBI", 0x11, 0x20, 31, 0, 4) + props
    if dt.kind == "S":
        return struct.pack("<BBBBI", 0x13, 0, 0, 0, size)
    raise H5Error(f"cannot write dtype {dt}")


def _space_msg(shape):
    return struct.pack("<BBBBI", 1, len(shape), 0, 0, 0) + b"".join(struct.pack("<Q", s) for s in shape)


def _msg(t, data, flags=0):
    data = data + b"\0" * (_pad8(len(data)) - len(data))
    return struct.pack("<HHB3x", t, len(data), flags) + data


class VlenStr(str):
    """A string attribute written as an HDF5 variable-length string (as h5py does)."""


class _Stored:
    """A dataset whose raw data is already in the file."""

    __slots__ = ("addr", "nbytes", "dtype", "shape", "attrs")

    def __init__(self, addr, nbytes, dtype, shape, attrs):
        self.addr, self.nbytes, self.dtype, self.shape, self.attrs = addr, nbytes, dtype, shape, attrs


class H5Writer:
    """Writes an HDF5 file: superblock 0, old-style groups, contiguous data.

    Dataset contents are appended to the file as `dataset()` is called; the
    object headers, group B-trees, heaps and the superblock are written by
    `close()`, so a large result series never has to sit in host memory."""

    LEAF_K = 4     # symbol-table node holds up to 2K entries
    INTERNAL_K = 16

    def __init__(self, path):
        self.path = path
        self.root = _Node()
        self.f = open(path, "wb")
        self.f.write(b"\0" * 96)  # superblock + root symbol-table entry, written at close
        self.pos = 96
        self._gheap = []  # (index, bytes) of variable-length string attributes

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _group(self, path, create=True):
        node = self.root
        for part in [p for p in path.split("/") if p]:
            nxt = node.children.get(part)
            if nxt is None:
                if not create:
                    raise KeyError(path)
                nxt = node.children[part] = _Node()
            if not isinstance(nxt, _Node):
                raise H5Error(f"{path}: '{part}' is a dataset")
            node = nxt
        return node

    def _append(self, data, align=8):
        pad = (-self.pos) % align
        if pad:
            self.f.write(b"\0" * pad)
            self.pos += pad
        a = self.pos
        self.f.write(data)
        self.pos += len(data)
        return a

    def dataset(self, path, data, attrs=None):
        """Create (or replace, as WriteData's H5Ldelete does) dataset `path`."""
        parts = [p for p in path.split("/") if p]
        g = self._group("/".join(parts[:-1]))
        arr = np.ascontiguousarray(data)
        if arr.dtype.byteorder == ">":
            arr = arr.astype(arr.dtype.newbyteorder("<"))
        addr = self._append(arr.tobytes()) if arr.nbytes else UNDEF
        g.children[parts[-1]] = _Stored(addr, arr.nbytes, arr.dtype, arr.shape if arr.ndim else (1,),
                                        dict(attrs or {}))

    def group_attrs(self, path, **attrs):
        self._group(path).attrs.update(attrs)

    def close(self):
        if self.f is None:
            return
        # variable-length strings live in one global heap collection; its address is
        # needed by the attribute messages, so it is placed first
        vl = []
        self._collect_vlen(self.root, vl)
        self._gheap_addr = UNDEF
        if vl:
            body = b""
            for i, txt in enumerate(vl, start=1):
                raw = txt.encode("utf-8")
                body += struct.pack("<HHIQ", i, 1, 0, len(raw)) + raw + b"\0" * (_pad8(len(raw)) - len(raw))
                self._gheap.append((i, txt))
            size = max(4096, 16 + len(body) + 16)
            free = size - 16 - len(body)
            body += struct.pack("<HHIQ", 0, 0, 0, free) + b"\0" * (free - 16)
            self._gheap_addr = self._append(b"GCOL" + bytes([1, 0, 0, 0]) + struct.pack("<Q", size) + body)
        root_addr = self._write_group(self.root)
        eof = self.pos
        sb = bytearray()
        sb += SIGNATURE
        sb += bytes([0, 0, 0, 0, 0, 8, 8, 0])
        sb += struct.pack("<HHI", self.LEAF_K, self.INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
        sb += struct.pack("<QQII", 0, root_addr, 0, 0) + b"\0" * 16
        self.f.seek(0)
        self.f.write(bytes(sb))
        self.f.close()
        self.f = None

    def _collect_vlen(self, node, out):
        items = node.children.values() if isinstance(node, _Node) else []
        for v in (node.attrs.values() if isinstance(node, _Node) else []):
            if isinstance(v, VlenStr):
                out.append(str(v))
        for ch in items:
            if isinstance(ch, _Node):
                self._collect_vlen(ch, out)
            else:
                out.extend(str(v) for v in ch.attrs.values() if isinstance(v, VlenStr))

    def _vlen_index(self, txt):
        for i, t in self._gheap:
            if t == txt:
                return i
        raise H5Error("variable-length string not in the global heap")

    def _attr_msgs(self, attrs):
        out = b""
        for k, v in attrs.items():
            if isinstance(v, VlenStr):
                name = k.encode() + b"\0"
                raw = str(v).encode("utf-8")
                base = struct.pack("<BBBBI", 0x10, 0, 0, 0, 1) + struct.pack("<HH", 0, 8)  # unsigned 8-bit char
                dt = struct.pack("<BBBBI", 0x19, 0x01, 0x01, 0, 16) + base  # vlen string, UTF-8
                sp = _space_msg(())
                body = struct.pack("<BBHHH", 1, 0, len(name), len(dt), len(sp))
                body += name + b"\0" * (_pad8(len(name)) - len(name))
                body += dt + b"\0" * (_pad8(len(dt)) - len(dt))
                body += sp + b"\0" * (_pad8(len(sp)) - len(sp))
                body += struct.pack("<IQI", len(raw), self._gheap_addr, self._vlen_index(str(v)))
                out += _msg(0x0C, body)
                continue
            if isinstance(v, str):
                v = np.frombuffer(v.encode() + b"\0", dtype=f"S{len(v.encode()) + 1}")[0]
            arr = np.asarray(v)
            name = k.encode() + b"\0"
            dt, sp = _dtype_msg(arr.dtype), _space_msg(arr.shape)  # rank 0: scalar
            body = struct.pack("<BBHHH", 1, 0, len(name), len(dt), len(sp))
            body += name + b"\0" * (_pad8(len(name)) - len(name))
            body += dt + b"\0" * (_pad8(len(dt)) - len(dt))
            body += sp + b"\0" * (_pad8(len(sp)) - len(sp))
            body += np.ascontiguousarray(arr).astype(arr.dtype.newbyteorder("<")).tobytes()
            out += _msg(0x0C, body)
        return out

    def _object_header(self, msgs, nmsg):
        hdr = struct.pack("<BBHII", 1, 0, nmsg, 1, len(msgs)) + b"\0" * 4
        return self._append(hdr + msgs)

    def _write_dataset(self, d):
        layout = struct.pack("<BBQQ", 3, 1, d.addr, d.nbytes)
        fill = struct.pack("<BBBB", 2, 2, 2, 0)  # fill value message v2: never written
        msgs = (_msg(0x01, _space_msg(d.shape)) + _msg(0x03, _dtype_msg(d.dtype), flags=1) + _msg(0x05, fill) +
                _msg(0x08, layout) + self._attr_msgs(d.attrs))
        return self._object_header(msgs, 4 + len(d.attrs))

    def _write_group(self, node):
        names = sorted(node.children, key=lambda s: s.encode())
        addrs = []
        for nm in names:
            ch = node.children[nm]
            addrs.append(self._write_group(ch) if isinstance(ch, _Node) else self._write_dataset(ch))
        # local heap: "" at 0, then the names
        heap = bytearray(b"\0" * 8)
        offs = []
        for nm in names:
            offs.append(len(heap))
            e = nm.encode() + b"\0"
            heap += e + b"\0" * (_pad8(len(e)) - len(e))
        heap_data = self._append(bytes(heap))
        heap_addr = self._append(b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap), UNDEF, heap_data))
        # symbol-table nodes of up to 2*LEAF_K entries, names in ascending order
        per = 2 * self.LEAF_K
        groups = [list(range(i, min(i + per, len(names)))) for i in range(0, len(names), per)] or [[]]
        if len(groups) > 2 * self.INTERNAL_K:
            raise H5Error(f"group with {len(names)} members: at most {2 * self.INTERNAL_K * per} supported")
        snods = []
        for grp in groups:
            body = b"SNOD" + struct.pack("<BBH", 1, 0, len(grp))
            for i in grp:
                body += struct.pack("<QQII", offs[i], addrs[i], 0, 0) + b"\0" * 16
            body += b"\0" * (40 * (per - len(grp)))
            snods.append(self._append(body))
        # one level-0 group B-tree node; key i+1 = heap offset of the last name in child i
        tree = b"TREE" + struct.pack("<BBHQQ", 0, 0, len(snods), UNDEF, UNDEF)
        tree += struct.pack("<Q", 0)
        for k, grp in enumerate(groups):
            last = offs[grp[-1]] if grp else 0
            tree += struct.pack("<QQ", snods[k], last)
        tree += b"\0" * ((2 * self.INTERNAL_K - len(snods)) * 16)
        tree_addr = self._append(tree)
        msgs = _msg(0x11, struct.pack("<QQ", tree_addr, heap_addr)) + self._attr_msgs(node.attrs)
        return self._object_header(msgs, 1 + len(node.attrs))
