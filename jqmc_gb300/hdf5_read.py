"""A minimal reader for the HDF5 files that TREXIO writes (no h5py needed).

It covers what those files use: superblock version 0 or 1, version-1 object
headers (with continuation blocks), groups held in version-1 B-trees with
local heaps, datasets stored compact, contiguous or chunked (version-1 chunk
B-tree, deflate and shuffle filters), fixed-point, floating-point and
fixed-length string types, and attributes.  It follows the published HDF5 File
Format Specification (superblock, object header messages 0x0001 dataspace,
0x0003 datatype, 0x0008 layout, 0x000B filter pipeline, 0x000C attribute,
0x0010 continuation, 0x0011 symbol table).  Other features raise
NotImplementedError.
"""

from __future__ import annotations

import struct
import zlib

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


def _pad8(n: int) -> int:
    return (n + 7) & ~7


class _Datatype:
    def __init__(self, buf: bytes, o: int):
        b0 = buf[o]
        self.cls = b0 & 0x0F
        bits = buf[o + 1] | (buf[o + 2] << 8) | (buf[o + 3] << 16)
        self.size = struct.unpack_from("<I", buf, o + 4)[0]
        order = ">" if bits & 1 else "<"
        if self.cls == 0:                      # fixed-point
            signed = bool(bits & 0x08)
            self.dtype = np.dtype(f"{order}{'i' if signed else 'u'}{self.size}")
        elif self.cls == 1:                    # floating-point
            self.dtype = np.dtype(f"{order}f{self.size}")
        elif self.cls == 3:                    # fixed-length string
            self.dtype = np.dtype(f"S{self.size}")
        elif self.cls == 9 and (bits & 0x0F) == 1:   # variable-length string (global heap references)
            self.dtype = np.dtype(object)
        else:
            self.dtype = None                  # (compound, other variable length, ...): not read


class _Dataspace:
    def __init__(self, buf: bytes, o: int, lsize: int):
        ver, rank, flags = buf[o], buf[o + 1], buf[o + 2]
        if ver == 1:
            p = o + 8
        elif ver == 2:
            p = o + 4
        else:
            raise NotImplementedError(f"dataspace version {ver}")
        self.shape = tuple(struct.unpack_from(f"<{rank}Q", buf, p)) if rank else ()


class Dataset:
    def __init__(self, f: "File", name: str, msgs: list):
        self.f, self.name = f, name
        self.dtype = self.space = self.layout = None
        self.filters = []
        self.attrs = {}
        buf = f.buf
        for mtype, o, size in msgs:
            if mtype == 0x0001:
                self.space = _Dataspace(buf, o, f.lsize)
            elif mtype == 0x0003:
                self.dtype = _Datatype(buf, o)
            elif mtype == 0x0008:
                self.layout = (o, size)
            elif mtype == 0x000B:
                self.filters = _filters(buf, o)
            elif mtype == 0x000C:
                k, v = _attribute(f, o)
                self.attrs[k] = v

    @property
    def shape(self):
        return self.space.shape

    def read(self) -> np.ndarray:
        if self.dtype is None or self.dtype.dtype is None:
            raise NotImplementedError(f"{self.name}: datatype class {self.dtype.cls if self.dtype else None}")
        buf, dt, shape = self.f.buf, self.dtype.dtype, self.space.shape
        n = int(np.prod(shape)) if shape else 1
        o, _ = self.layout
        if dt == np.dtype(object):   # variable-length strings, contiguous: (length, heap address, index) per element
            if buf[o] != 3 or buf[o + 1] != 1:
                raise NotImplementedError(f"{self.name}: variable-length strings outside contiguous storage")
            addr = struct.unpack_from("<Q", buf, o + 2)[0]
            out = np.empty(n, dtype=object)
            for i in range(n):
                _, gcol, idx = struct.unpack_from("<IQI", buf, addr + 16 * i)
                out[i] = self.f._global_heap_object(gcol, idx).decode()
            return out.reshape(shape)
        ver = buf[o]
        if ver != 3:
            raise NotImplementedError(f"{self.name}: layout message version {ver}")
        cls = buf[o + 1]
        if cls == 0:                                   # compact
            size = struct.unpack_from("<H", buf, o + 2)[0]
            raw = buf[o + 4:o + 4 + size]
            return np.frombuffer(raw, dtype=dt, count=n).reshape(shape).copy()
        if cls == 1:                                   # contiguous
            addr, size = struct.unpack_from("<QQ", buf, o + 2)
            if addr == _UNDEF:
                return np.zeros(shape, dtype=dt)
            return np.frombuffer(buf, dtype=dt, count=n, offset=addr).reshape(shape).copy()
        if cls == 2:                                   # chunked
            nd = buf[o + 2]
            btree = struct.unpack_from("<Q", buf, o + 3)[0]
            cdims = struct.unpack_from(f"<{nd}I", buf, o + 11)[:-1]
            out = np.zeros(shape, dtype=dt)
            if btree != _UNDEF:
                for offs, addr, csize, mask in self.f._chunks(btree, nd):
                    raw = bytes(buf[addr:addr + csize])
                    raw = _unfilter(raw, self.filters, mask, dt.itemsize)
                    chunk = np.frombuffer(raw, dtype=dt, count=int(np.prod(cdims))).reshape(cdims)
                    sl = tuple(slice(a, min(a + c, s)) for a, c, s in zip(offs, cdims, shape))
                    out[sl] = chunk[tuple(slice(0, s.stop - s.start) for s in sl)]
            return out
        raise NotImplementedError(f"{self.name}: layout class {cls}")


class Group:
    def __init__(self, f: "File", name: str, btree: int, heap: int, msgs: list):
        self.f, self.name = f, name
        self.attrs = {}
        for mtype, o, _ in msgs:
            if mtype == 0x000C:
                k, v = _attribute(f, o)
                self.attrs[k] = v
        self._entries = f._group_entries(btree, heap)

    def keys(self):
        return list(self._entries)

    def __contains__(self, k):
        return k in self._entries

    def __getitem__(self, path: str):
        head, _, rest = path.partition("/")
        obj = self.f._object(self._entries[head], f"{self.name}/{head}")
        return obj[rest] if rest else obj


class File:
    """Read-only view of an HDF5 file held in memory."""

    def __init__(self, path: str):
        with open(path, "rb") as fh:
            self.buf = memoryview(fh.read())
        buf = self.buf
        if bytes(buf[:8]) != _SIG:
            raise ValueError(f"{path}: not an HDF5 file")
        ver = buf[8]
        if ver not in (0, 1):
            raise NotImplementedError(f"superblock version {ver}")
        self.osize, self.lsize = buf[13], buf[14]
        if (self.osize, self.lsize) != (8, 8):
            raise NotImplementedError("offsets and lengths other than 8 bytes")
        p = 24 if ver == 0 else 28
        p += 4 * 8                       # base, free-space, end-of-file, driver addresses
        ohdr = struct.unpack_from("<Q", buf, p + 8)[0]
        self.root = self._object(ohdr, "")

    def __getitem__(self, path: str):
        return self.root[path.strip("/")]

    def keys(self):
        return self.root.keys()

    # ------------------------------------------------------------ object headers
    def _messages(self, addr: int) -> list:
        buf = self.buf
        if buf[addr] != 1:
            raise NotImplementedError(f"object header version {buf[addr]}")
        nmsg = struct.unpack_from("<H", buf, addr + 2)[0]
        hsize = struct.unpack_from("<I", buf, addr + 8)[0]
        blocks = [(addr + 16, hsize)]
        msgs = []
        while blocks and len(msgs) < nmsg:
            p, size = blocks.pop(0)
            end = p + size
            while p + 8 <= end and len(msgs) < nmsg:
                mtype, msize = struct.unpack_from("<HH", buf, p)
                data = p + 8
                if mtype == 0x0010:
                    blocks.append(struct.unpack_from("<QQ", buf, data))
                msgs.append((mtype, data, msize))
                p = data + msize
        return msgs

    def _object(self, addr: int, name: str):
        msgs = self._messages(addr)
        for mtype, o, _ in msgs:
            if mtype == 0x0011:
                btree, heap = struct.unpack_from("<QQ", self.buf, o)
                return Group(self, name, btree, heap, msgs)
        return Dataset(self, name, msgs)

    def _global_heap_object(self, gcol: int, index: int) -> bytes:
        """Object ``index`` of the global heap collection at ``gcol``."""
        buf = self.buf
        if bytes(buf[gcol:gcol + 4]) != b"GCOL":
            raise ValueError("bad global heap collection")
        size = struct.unpack_from("<Q", buf, gcol + 8)[0]
        p, end = gcol + 16, gcol + size
        while p + 16 <= end:
            idx, _, osize = struct.unpack_from("<HH4xQ", buf, p)
            if idx == 0:
                break
            if idx == index:
                return bytes(buf[p + 16:p + 16 + osize])
            p += 16 + _pad8(osize)
        raise KeyError(f"global heap object {index}")

    # ------------------------------------------------------------ groups
    def _heap_data(self, heap: int) -> int:
        if bytes(self.buf[heap:heap + 4]) != b"HEAP":
            raise ValueError("bad local heap")
        return struct.unpack_from("<Q", self.buf, heap + 24)[0]

    def _name(self, heap_data: int, off: int) -> str:
        buf = self.buf
        p = heap_data + off
        e = p
        while buf[e] != 0:
            e += 1
        return bytes(buf[p:e]).decode()

    def _group_entries(self, btree: int, heap: int) -> dict:
        hd = self._heap_data(heap)
        out = {}
        for snod in self._btree_children(btree, 0):
            buf = self.buf
            if bytes(buf[snod:snod + 4]) != b"SNOD":
                raise ValueError("bad symbol node")
            nsym = struct.unpack_from("<H", buf, snod + 6)[0]
            for i in range(nsym):
                e = snod + 8 + 40 * i
                name_off, ohdr = struct.unpack_from("<QQ", buf, e)
                out[self._name(hd, name_off)] = ohdr
        return out

    def _btree_children(self, node: int, ntype: int, nd: int = 0):
        """Leaf children of a version-1 B-tree (group nodes: symbol-node addresses)."""
        buf = self.buf
        if bytes(buf[node:node + 4]) != b"TREE" or buf[node + 4] != ntype:
            raise ValueError("bad B-tree node")
        level = buf[node + 5]
        used = struct.unpack_from("<H", buf, node + 6)[0]
        ksize = 8 if ntype == 0 else 8 + 8 * nd
        p = node + 24
        for i in range(used):
            child = struct.unpack_from("<Q", buf, p + ksize)[0]
            if level == 0:
                yield child
            else:
                yield from self._btree_children(child, ntype, nd)
            p += ksize + 8

    def _chunks(self, node: int, nd: int):
        """(chunk offsets, address, stored size, filter mask) of a chunked dataset."""
        buf = self.buf
        if bytes(buf[node:node + 4]) != b"TREE" or buf[node + 4] != 1:
            raise ValueError("bad chunk B-tree node")
        level = buf[node + 5]
        used = struct.unpack_from("<H", buf, node + 6)[0]
        ksize = 8 + 8 * nd
        p = node + 24
        for i in range(used):
            csize, mask = struct.unpack_from("<II", buf, p)
            offs = struct.unpack_from(f"<{nd}Q", buf, p + 8)[:-1]
            child = struct.unpack_from("<Q", buf, p + ksize)[0]
            if level == 0:
                yield offs, child, csize, mask
            else:
                yield from self._chunks(child, nd)
            p += ksize + 8


def _filters(buf, o: int) -> list:
    ver, nf = buf[o], buf[o + 1]
    out = []
    p = o + (8 if ver == 1 else 2)
    for _ in range(nf):
        fid = struct.unpack_from("<H", buf, p)[0]
        if ver == 1 or fid >= 256:
            nlen = struct.unpack_from("<H", buf, p + 2)[0]
            flags, nval = struct.unpack_from("<HH", buf, p + 4)
            p += 8 + (_pad8(nlen) if ver == 1 else nlen)
        else:
            nlen = 0
            flags, nval = struct.unpack_from("<HH", buf, p + 2)
            p += 6
        vals = struct.unpack_from(f"<{nval}I", buf, p)
        p += 4 * nval + (4 if ver == 1 and nval % 2 else 0)
        out.append((fid, vals))
    return out


def _unfilter(raw: bytes, filters: list, mask: int, itemsize: int) -> bytes:
    for i, (fid, _) in reversed(list(enumerate(filters))):
        if mask & (1 << i):
            continue
        if fid == 1:
            raw = zlib.decompress(raw)
        elif fid == 2:
            a = np.frombuffer(raw, dtype=np.uint8)
            raw = a.reshape(itemsize, -1).T.copy().tobytes()
        else:
            raise NotImplementedError(f"filter {fid}")
    return raw


def _attribute(f: File, o: int):
    buf = f.buf
    ver = buf[o]
    nsize, tsize, ssize = struct.unpack_from("<HHH", buf, o + 2)
    if ver == 1:
        p = o + 8
        name = bytes(buf[p:p + nsize - 1]).decode()
        p += _pad8(nsize)
        dt = _Datatype(buf, p)
        p += _pad8(tsize)
        sp = _Dataspace(buf, p, f.lsize)
        p += _pad8(ssize)
    elif ver in (2, 3):
        p = o + 8 + (1 if ver == 3 else 0)
        name = bytes(buf[p:p + nsize - 1]).decode()
        p += nsize
        dt = _Datatype(buf, p)
        p += tsize
        sp = _Dataspace(buf, p, f.lsize)
        p += ssize
    else:
        raise NotImplementedError(f"attribute message version {ver}")
    if dt.dtype is None:
        return name, None
    n = int(np.prod(sp.shape)) if sp.shape else 1
    val = np.frombuffer(buf, dtype=dt.dtype, count=n, offset=p).reshape(sp.shape).copy()
    return name, (val[()] if val.shape == () else val)
