"""Minimal NetCDF classic (CDF-1 / CDF-2 "64-bit offset") reader and writer.

The reference reads its Exodus meshes and writes its station output through NetCDF-C
(SOLVER/src/preloop/utilities/NetCDF_Reader.*, NetCDF_Writer.h:19-185).  No NetCDF or HDF5
library exists here, so this module implements the classic file format from its published
specification: header (magic, numrecs, dimension list, global attributes, variable list
with begin offsets) followed by big-endian, 4-byte-padded data.  Only fixed-size (non
record) variables are written; the reader also accepts record variables of one record.
NetCDF-4 / HDF5 files (magic "\\x89HDF", the format of AxiSEM3D's own meshes) go to the
HDF5 reader of `hdf5.py`.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

NC_DIMENSION, NC_VARIABLE, NC_ATTRIBUTE = 0x0A, 0x0B, 0x0C
TYPES = {1: ">i1", 2: "S1", 3: ">i2", 4: ">i4", 5: ">f4", 6: ">f8"}
CODES = {np.dtype(">i1"): 1, np.dtype("S1"): 2, np.dtype(">i2"): 3, np.dtype(">i4"): 4,
         np.dtype(">f4"): 5, np.dtype(">f8"): 6}


def _pad4(n: int) -> int:
    return (4 - n % 4) % 4


@dataclass
class Variable:
    name: str
    dims: tuple
    data: np.ndarray
    attrs: dict = field(default_factory=dict)


class Dataset:
    """In-memory NetCDF dataset: dims {name: size}, variables {name: Variable}, attrs."""

    def __init__(self):
        self.dims: dict[str, int] = {}
        self.variables: dict[str, Variable] = {}
        self.attrs: dict = {}

    # ---------------------------------------------------------------- building
    def add_dim(self, name: str, size: int):
        if name in self.dims and self.dims[name] != size:
            raise ValueError(f"dimension {name} redefined")
        self.dims[name] = int(size)

    def add_var(self, name: str, dims, data, attrs=None, dtype=None):
        data = np.asarray(data)
        if dtype is not None:
            data = data.astype(dtype)
        if data.dtype.kind == "f" and data.dtype.itemsize == 4:
            data = data.astype(">f4")
        elif data.dtype.kind == "f":
            data = data.astype(">f8")
        elif data.dtype.kind in "iu":
            data = data.astype(">i4")
        elif data.dtype.kind == "S":
            data = data.astype("S1")
        dims = tuple(dims)
        shape = tuple(self.dims[d] for d in dims)
        if data.shape != shape:
            raise ValueError(f"{name}: shape {data.shape} != dims {shape}")
        self.variables[name] = Variable(name, dims, data, dict(attrs or {}))

    def add_strings(self, name: str, dim_n: str, dim_len: str, strings, length: int = 33):
        self.add_dim(dim_n, len(strings))
        self.add_dim(dim_len, length)
        arr = np.zeros((len(strings), length), "S1")
        for i, s in enumerate(strings):
            b = s.encode()[:length - 1]
            arr[i, :len(b)] = np.frombuffer(b, "S1")
        self.add_var(name, (dim_n, dim_len), arr)

    def strings(self, name: str):
        a = self.variables[name].data
        return [b"".join(row).split(b"\0")[0].decode().strip() for row in a]

    def __getitem__(self, name):
        return self.variables[name].data

    def __contains__(self, name):
        return name in self.variables


# -------------------------------------------------------------------- writing
def _name(b: bytearray, s: str):
    e = s.encode()
    b += struct.pack(">i", len(e)) + e + b"\0" * _pad4(len(e))


def _attrs(b: bytearray, attrs: dict):
    if not attrs:
        b += struct.pack(">ii", 0, 0)
        return
    b += struct.pack(">ii", NC_ATTRIBUTE, len(attrs))
    for k, v in attrs.items():
        _name(b, k)
        if isinstance(v, str):
            e = v.encode()
            b += struct.pack(">ii", 2, len(e)) + e + b"\0" * _pad4(len(e))
        else:
            a = np.atleast_1d(np.asarray(v))
            a = a.astype(">f8") if a.dtype.kind == "f" else a.astype(">i4")
            raw = a.tobytes()
            b += struct.pack(">ii", CODES[a.dtype], a.size) + raw + b"\0" * _pad4(len(raw))


def write(path, ds: Dataset):
    """Write ds as CDF-2 (64-bit offsets)."""
    dims = list(ds.dims.items())
    dim_index = {n: i for i, (n, _) in enumerate(dims)}

    def header(begins):
        b = bytearray(b"CDF\x02")
        b += struct.pack(">i", 0)
        if dims:
            b += struct.pack(">ii", NC_DIMENSION, len(dims))
            for n, sz in dims:
                _name(b, n)
                b += struct.pack(">i", sz)
        else:
            b += struct.pack(">ii", 0, 0)
        _attrs(b, ds.attrs)
        vs = list(ds.variables.values())
        if vs:
            b += struct.pack(">ii", NC_VARIABLE, len(vs))
            for v, beg in zip(vs, begins):
                _name(b, v.name)
                b += struct.pack(">i", len(v.dims))
                for d in v.dims:
                    b += struct.pack(">i", dim_index[d])
                _attrs(b, v.attrs)
                nbytes = v.data.nbytes
                b += struct.pack(">iiq", CODES[v.data.dtype], nbytes + _pad4(nbytes), beg)
        else:
            b += struct.pack(">ii", 0, 0)
        return b

    vs = list(ds.variables.values())
    hlen = len(header([0] * len(vs)))
    begins, pos = [], hlen
    for v in vs:
        begins.append(pos)
        pos += v.data.nbytes + _pad4(v.data.nbytes)
    with open(path, "wb") as f:
        f.write(header(begins))
        for v in vs:
            raw = np.ascontiguousarray(v.data).tobytes()
            f.write(raw + b"\0" * _pad4(len(raw)))


# -------------------------------------------------------------------- reading
class _Reader:
    def __init__(self, buf: bytes):
        self.b = buf
        self.p = 0

    def i4(self):
        v = struct.unpack_from(">i", self.b, self.p)[0]
        self.p += 4
        return v

    def i8(self):
        v = struct.unpack_from(">q", self.b, self.p)[0]
        self.p += 8
        return v

    def name(self):
        n = self.i4()
        s = self.b[self.p:self.p + n].decode()
        self.p += n + _pad4(n)
        return s

    def attrs(self):
        tag, n = self.i4(), self.i4()
        out = {}
        for _ in range(n if tag == NC_ATTRIBUTE else 0):
            k = self.name()
            t, cnt = self.i4(), self.i4()
            dt = np.dtype(TYPES[t])
            nb = cnt * dt.itemsize
            raw = self.b[self.p:self.p + nb]
            self.p += nb + _pad4(nb)
            out[k] = raw.decode(errors="replace").rstrip("\0") if t == 2 else np.frombuffer(raw, dt).copy()
        return out


def read(path) -> Dataset:
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:4] == b"\x89HDF":
        from . import hdf5
        return hdf5.read(path)
    if buf[:3] != b"CDF" or buf[3] not in (1, 2):
        raise ValueError(f"{path}: not a NetCDF classic file")
    version = buf[3]
    r = _Reader(buf)
    r.p = 4
    numrecs = r.i4()
    ds = Dataset()
    tag, n = r.i4(), r.i4()
    dims = []
    for _ in range(n if tag == NC_DIMENSION else 0):
        nm = r.name()
        sz = r.i4()
        dims.append((nm, sz))
        ds.dims[nm] = sz if sz else numrecs
    ds.attrs = r.attrs()
    tag, n = r.i4(), r.i4()
    for _ in range(n if tag == NC_VARIABLE else 0):
        nm = r.name()
        nd = r.i4()
        ids = [r.i4() for _ in range(nd)]
        at = r.attrs()
        t = r.i4()
        r.i4()  # vsize
        beg = r.i8() if version == 2 else r.i4()
        dt = np.dtype(TYPES[t])
        shape = tuple(ds.dims[dims[i][0]] for i in ids)
        cnt = int(np.prod(shape)) if shape else 1
        data = np.frombuffer(buf, dt, cnt, beg).reshape(shape)
        ds.variables[nm] = Variable(nm, tuple(dims[i][0] for i in ids), data.copy(), at)
    return ds
