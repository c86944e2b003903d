"""Minimal reader for NetCDF-4 files stored in HDF5 (the format AxiSEM3D's meshes use).

The reference opens its Exodus meshes through NetCDF-C, which reads NetCDF-4 / HDF5 files
(SOLVER/src/preloop/utilities/NetCDF_Reader.cpp:15).  No HDF5 library exists here, so this
module implements the part of the published HDF5 file format (version 0 / 1 superblock)
that such files use: object headers of version 1, groups held in symbol tables (version 1
B-trees of type 0, symbol-table nodes, local heaps), datasets with compact, contiguous or
chunked layout (version 1 B-trees of type 1), the deflate, shuffle and Fletcher-32 filters,
and fixed-point, floating-point and fixed-length string datatypes.  Every dataset of the
root group becomes a variable of a `netcdf.Dataset`; attributes are not read.  A file
outside that subset raises ValueError; a dataset outside it (variable-length strings, shared
messages) is left out and named in the dataset's attrs["unread_datasets"].
"""
from __future__ import annotations

import zlib

import numpy as np

from .netcdf import Dataset, Variable

MAGIC = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class _File:
    def __init__(self, buf: bytes):
        self.b = buf
        if buf[:8] != MAGIC:
            raise ValueError("HDF5 || bad signature")
        ver = buf[8]
        if ver not in (0, 1):
            raise ValueError(f"HDF5 || superblock version {ver} is not supported (0 or 1 only)")
        self.so, self.sl = buf[13], buf[14]
        if self.so != 8 or self.sl != 8:
            raise ValueError("HDF5 || only 8-byte offsets and lengths are supported")
        p = 24 + (4 if ver == 1 else 0)
        self.base = self.u(p, 8)
        p += 4 * 8  # base, free-space, end-of-file, driver block addresses
        self.root = self.entry(p)

    def u(self, p, n):
        return int.from_bytes(self.b[p:p + n], "little")

    def entry(self, p):
        """Symbol table entry: (link name offset, object header address, B-tree, heap)."""
        name_off, ohdr = self.u(p, 8), self.u(p + 8, 8)
        cache = self.u(p + 16, 4)
        bt = hp = None
        if cache == 1:
            bt, hp = self.u(p + 24, 8), self.u(p + 32, 8)
        return name_off, ohdr, bt, hp

    # ------------------------------------------------------------ object headers
    def messages(self, addr):
        """(type, data bytes) of every message of the version-1 object header at addr."""
        b = self.b
        if b[addr] != 1:
            raise ValueError(f"HDF5 || object header version {b[addr]} is not supported")
        nmsg = self.u(addr + 2, 2)
        size = self.u(addr + 8, 4)
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            p, n = blocks.pop(0)
            end = p + n
            while p + 8 <= end and len(out) < nmsg:
                mt, ms, flags = self.u(p, 2), self.u(p + 2, 2), b[p + 4]
                data = b[p + 8:p + 8 + ms]
                if flags & 0x02 and mt in (0x01, 0x03, 0x05, 0x08, 0x0B):
                    raise ValueError(f"HDF5 || shared header message (type {mt}) is not supported")
                p += 8 + ms
                if mt == 0x10:  # continuation
                    blocks.append((int.from_bytes(data[0:8], "little"), int.from_bytes(data[8:16], "little")))
                out.append((mt, data))
        return out

    # -------------------------------------------------------------------- groups
    def group(self, bt, hp):
        """{name: object header address} of a symbol-table group."""
        if self.b[hp:hp + 4] != b"HEAP":
            raise ValueError("HDF5 || bad local heap")
        heap = self.u(hp + 24, 8)
        out = {}
        for snod in self._btree_children(bt, 0):
            if self.b[snod:snod + 4] != b"SNOD":
                raise ValueError("HDF5 || bad symbol table node")
            n = self.u(snod + 6, 2)
            for i in range(n):
                name_off, ohdr, _, _ = self.entry(snod + 8 + 40 * i)
                s = heap + name_off
                name = self.b[s:self.b.index(b"\0", s)].decode()
                out[name] = ohdr
        return out

    def _btree_children(self, addr, ntype, ndims=0):
        """Leaf children (addresses; with their keys for chunk trees) of a version-1 B-tree."""
        b = self.b
        if b[addr:addr + 4] != b"TREE" or b[addr + 4] != ntype:
            raise ValueError("HDF5 || bad B-tree node")
        level, used = b[addr + 5], self.u(addr + 6, 2)
        ksize = 8 if ntype == 0 else 8 + 8 * ndims
        p = addr + 24
        out = []
        for i in range(used):
            key = b[p:p + ksize]
            child = self.u(p + ksize, 8)
            p += ksize + 8
            if level > 0:
                out.extend(self._btree_children(child, ntype, ndims))
            else:
                out.append(child if ntype == 0 else (key, child))
        return out

    # ------------------------------------------------------------------ datasets
    def dataset(self, addr):
        shape = dtype = layout = None
        filters = []
        for mt, d in self.messages(addr):
            if mt == 0x01:
                shape = self._dataspace(d)
            elif mt == 0x03:
                dtype = self._datatype(d)
            elif mt == 0x08:
                layout = d
            elif mt == 0x0B:
                filters = self._filters(d)
        if shape is None or dtype is None or layout is None:
            return None
        n = int(np.prod(shape)) if shape else 1
        raw = self._read_layout(layout, shape, dtype, filters)
        return np.frombuffer(raw, dtype, n).reshape(shape).copy()

    @staticmethod
    def _dataspace(d):
        ver, nd, flags = d[0], d[1], d[2]
        p = 8 if ver == 1 else 4
        if ver == 2 and d[3] == 2:  # null dataspace
            return None
        return tuple(int.from_bytes(d[p + 8 * i:p + 8 * i + 8], "little") for i in range(nd))

    @staticmethod
    def _datatype(d):
        cls, bits, size = d[0] & 0x0F, d[1], int.from_bytes(d[4:8], "little")
        order = ">" if bits & 1 else "<"
        if cls == 0:
            return np.dtype(f"{order}{'i' if bits & 8 else 'u'}{size}")
        if cls == 1:
            return np.dtype(f"{order}f{size}")
        if cls == 3:
            return np.dtype(f"S{size}")
        raise ValueError(f"HDF5 || datatype class {cls} is not supported")

    @staticmethod
    def _filters(d):
        ver, nf = d[0], d[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(nf):
            fid = int.from_bytes(d[p:p + 2], "little")
            if ver == 1 or fid >= 256:
                nlen = int.from_bytes(d[p + 2:p + 4], "little")
                p += 2
            else:
                nlen = 0
            nval = int.from_bytes(d[p + 4:p + 6], "little")
            p += 6
            if ver == 1:
                nlen = (nlen + 7) // 8 * 8
            p += nlen
            vals = [int.from_bytes(d[p + 4 * i:p + 4 * i + 4], "little") for i in range(nval)]
            p += 4 * nval
            if ver == 1 and nval % 2:
                p += 4
            out.append((fid, vals))
        return out

    def _unfilter(self, raw, filters, mask, itemsize):
        for i in range(len(filters) - 1, -1, -1):
            fid, _ = filters[i]
            if mask & (1 << i):
                continue
            if fid == 1:
                raw = zlib.decompress(raw)
            elif fid == 2:
                n = len(raw) // itemsize
                raw = np.frombuffer(raw[:n * itemsize], np.uint8).reshape(itemsize, n).T.tobytes()
            elif fid == 3:
                raw = raw[:-4]
            else:
                raise ValueError(f"HDF5 || filter {fid} is not supported")
        return raw

    def _read_layout(self, d, shape, dtype, filters):
        ver = d[0]
        nbytes = (int(np.prod(shape)) if shape else 1) * dtype.itemsize
        if ver == 3:
            cls = d[1]
            if cls == 0:
                size = int.from_bytes(d[2:4], "little")
                return d[4:4 + size]
            if cls == 1:
                a = int.from_bytes(d[2:10], "little")
                if a == UNDEF:
                    return bytes(nbytes)
                return self.b[a:a + nbytes]
            if cls == 2:
                nd = d[2]
                bt = int.from_bytes(d[3:11], "little")
                cdims = [int.from_bytes(d[11 + 4 * i:15 + 4 * i], "little") for i in range(nd)]
                return self._chunked(bt, shape, cdims[:-1], dtype, filters)
        elif ver in (1, 2):
            nd, cls = d[1], d[2]
            a = int.from_bytes(d[8:16], "little") if cls != 0 else None
            cdims = [int.from_bytes(d[16 + 4 * i:20 + 4 * i], "little") for i in range(nd)]
            if cls == 1:
                return self.b[a:a + nbytes]
            if cls == 2:
                return self._chunked(a, shape, cdims[:-1], dtype, filters)
            if cls == 0:
                p = 16 + 4 * nd
                size = int.from_bytes(d[p:p + 4], "little")
                return d[p + 4:p + 4 + size]
        raise ValueError(f"HDF5 || data layout version {ver} is not supported")

    def _chunked(self, bt, shape, cdims, dtype, filters):
        out = np.zeros(shape, dtype)
        if bt == UNDEF:
            return out.tobytes()
        nd = len(shape)
        for key, addr in self._btree_children(bt, 1, nd + 1):
            csize = int.from_bytes(key[0:4], "little")
            mask = int.from_bytes(key[4:8], "little")
            offs = [int.from_bytes(key[8 + 8 * i:16 + 8 * i], "little") for i in range(nd)]
            raw = self._unfilter(self.b[addr:addr + csize], filters, mask, dtype.itemsize)
            chunk = np.frombuffer(raw, dtype, int(np.prod(cdims))).reshape(cdims)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
            out[sl] = chunk[tuple(slice(0, x.stop - x.start) for x in sl)]
        return out.tobytes()


def read(path) -> Dataset:
    """Every dataset of the root group of a NetCDF-4 / HDF5 file as a netcdf.Dataset
    (string datasets of one byte per element become 'S1' arrays, as NetCDF char data)."""
    with open(path, "rb") as f:
        buf = f.read()
    h = _File(buf)
    _, ohdr, bt, hp = h.root
    if bt is None:
        for mt, d in h.messages(ohdr):
            if mt == 0x11:
                bt, hp = int.from_bytes(d[0:8], "little"), int.from_bytes(d[8:16], "little")
    if bt is None:
        raise ValueError("HDF5 || the root group has no symbol table (newer group format)")
    ds = Dataset()
    unread = []
    for name, addr in h.group(bt, hp).items():
        try:
            data = h.dataset(addr)
        except ValueError:  # a dataset outside the subset (e.g. variable-length strings)
            unread.append(name)
            continue
        if data is None:
            continue
        if data.dtype.kind == "S" and data.dtype.itemsize == 1:
            data = data.astype("S1")
        dims = tuple(f"{name}_d{i}" for i in range(data.ndim))
        for dn, n in zip(dims, data.shape):
            ds.dims[dn] = n
        ds.variables[name] = Variable(name, dims, data, {})
    ds.attrs["unread_datasets"] = unread
    return ds
