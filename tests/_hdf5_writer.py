"""Test infrastructure: a minimal writer of the HDF5 subset `axisem3d_gb300.hdf5` reads
(version 0 superblock, one root group held in a symbol table, version 1 object headers,
compact and contiguous datasets, chunked datasets through the shuffle, deflate and
Fletcher-32 filters), so that the reader is exercised without an HDF5 library or an
external file.  Written from the published HDF5 format specification; little-endian int32 /
float64 and one-byte strings only."""
from __future__ import annotations

import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * (-len(b) % 8)


def _msg(mtype: int, data: bytes) -> bytes:
    data = _pad8(data)
    return struct.pack("<HHB3x", mtype, len(data), 0) + data


def _ohdr(msgs: list) -> bytes:
    body = b"".join(msgs)
    return struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(body)) + body


def _datatype(a: np.ndarray) -> bytes:
    if a.dtype == np.dtype("<i4"):
        return struct.pack("<B3sI", 0x10 | 0, bytes([0x08, 0, 0]), 4) + struct.pack("<HH", 0, 32)
    if a.dtype == np.dtype("<f8"):
        return struct.pack("<B3sI", 0x10 | 1, bytes([0x20, 0x3F, 0]), 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0,
                                                                                     52, 1023)
    if a.dtype == np.dtype("S1"):
        return struct.pack("<B3sI", 0x10 | 3, bytes([0, 0, 0]), 1)
    raise ValueError(f"unsupported dtype {a.dtype}")


def _fletcher32(b: bytes) -> int:
    """Fletcher-32 over little-endian 16-bit words (an odd last byte padded with zero)."""
    if len(b) % 2:
        b += b"\0"
    s1 = s2 = 0
    for (w,) in struct.iter_unpack("<H", b):
        s1 = (s1 + w) % 65535
        s2 = (s2 + s1) % 65535
    return (s2 << 16) | s1


def _filter_message(filters, itemsize) -> bytes:
    """Filter pipeline message, version 1: (id, name length 0, flags 0, client values)."""
    ids = {"shuffle": (2, [itemsize]), "deflate": (1, [6]), "fletcher32": (3, [])}
    body = b""
    for f in filters:
        fid, vals = ids[f]
        body += struct.pack("<HHHH", fid, 0, 0, len(vals)) + b"".join(struct.pack("<I", v) for v in vals)
        body += b"\0" * (4 * (len(vals) % 2))
    return struct.pack("<BB6x", 1, len(filters)) + body


def _apply_filters(raw: bytes, filters, itemsize) -> bytes:
    for f in filters:
        if f == "shuffle":
            raw = np.frombuffer(raw, np.uint8).reshape(-1, itemsize).T.tobytes()
        elif f == "deflate":
            raw = zlib.compress(raw)
        else:
            raw = raw + struct.pack("<I", _fletcher32(raw))
    return raw


def _chunk_key(size, corner) -> bytes:
    return struct.pack("<II", size, 0) + b"".join(struct.pack("<Q", int(o)) for o in corner) + struct.pack("<Q", 0)


def _chunk_tree(keys, shape, put, fanout) -> int:
    """Version 1 B-tree of chunks: one leaf node, or (fanout > 0) leaves of at most fanout
    chunks under a level-1 root; returns the root's address."""
    end = _chunk_key(0, shape)

    def node(level, entries):
        b = bytearray(b"TREE" + bytes([1, level]) + struct.pack("<HQQ", len(entries), UNDEF, UNDEF))
        for key, addr in entries:
            b += key + struct.pack("<Q", addr)
        return bytes(b + end)
    leaf_entries = [(_chunk_key(size, corner), addr) for size, corner, addr in keys]
    if not fanout or len(leaf_entries) <= fanout:
        return put(node(0, leaf_entries))
    leaves = [leaf_entries[i:i + fanout] for i in range(0, len(leaf_entries), fanout)]
    return put(node(1, [(lf[0][0], put(node(0, lf))) for lf in leaves]))


def write(path, datasets: dict, fanout: int = 0, continuation: bool = False):
    """datasets: name -> array (contiguous), (array, "compact"), (array, chunk shape) for a
    chunked, deflated dataset, or (array, chunk shape, filters) with filters a sequence of
    "shuffle", "deflate" and "fletcher32" in the order they are applied.  fanout > 0: chunk
    B-trees of two levels, at most fanout chunks per leaf; continuation: every dataset's
    object header keeps its first two messages and continues in a second block."""
    out = bytearray(b"\0" * 96)  # superblock, written last
    names = sorted(datasets)
    # local heap data: "" at offset 0, then the names, each padded to 8 bytes
    heap_data = bytearray(b"\0" * 8)
    offs = {}
    for n in names:
        offs[n] = len(heap_data)
        heap_data += _pad8(n.encode() + b"\0")

    def put(b: bytes) -> int:
        addr = len(out)
        out.extend(b)
        out.extend(b"\0" * (-len(out) % 8))
        return addr

    heap_data_addr = put(bytes(heap_data))
    heap_addr = put(b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap_data), UNDEF, heap_data_addr))
    ohdr = {}
    for n in names:
        spec = datasets[n] if isinstance(datasets[n], tuple) else (datasets[n],)
        a, chunks = spec[0], (spec[1] if len(spec) > 1 else None)
        filters = spec[2] if len(spec) > 2 else ("deflate",)
        a = np.ascontiguousarray(a)
        nd = a.ndim
        space = struct.pack("<BBBB4x", 1, nd, 0, 0) + b"".join(struct.pack("<Q", d) for d in a.shape)
        msgs = [_msg(0x01, space), _msg(0x03, _datatype(a))]
        if chunks == "compact":
            msgs.append(_msg(0x08, struct.pack("<BBH", 3, 0, a.nbytes) + a.tobytes()))
        elif chunks is None:
            addr = put(a.tobytes())
            msgs.append(_msg(0x08, struct.pack("<BBQQ", 3, 1, addr, a.nbytes)))
        else:
            keys = []
            grid = [range(0, s, c) for s, c in zip(a.shape, chunks)]
            for corner in np.array(np.meshgrid(*grid, indexing="ij")).reshape(nd, -1).T:
                block = np.zeros(chunks, a.dtype)
                sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(corner, chunks, a.shape))
                block[tuple(slice(0, x.stop - x.start) for x in sl)] = a[sl]
                raw = _apply_filters(block.tobytes(), filters, a.itemsize)
                keys.append((len(raw), corner, put(raw)))
            bt = _chunk_tree(keys, a.shape, put, fanout)
            msgs.append(_msg(0x08, struct.pack("<BBBQ", 3, 2, nd + 1, bt) +
                             b"".join(struct.pack("<I", c) for c in chunks) + struct.pack("<I", a.itemsize)))
            msgs.append(_msg(0x0B, _filter_message(filters, a.itemsize)))
        if continuation and len(msgs) > 2:
            rest = b"".join(msgs[2:])
            caddr = put(rest)
            cont = _msg(0x10, struct.pack("<QQ", caddr, len(rest)))
            body = b"".join(msgs[:2]) + cont
            ohdr[n] = put(struct.pack("<BBHII4x", 1, 0, len(msgs) + 1, 1, len(body)) + body)
        else:
            ohdr[n] = put(_ohdr(msgs))
    snod = bytearray(b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(names)))
    for n in names:
        snod += struct.pack("<QQII16x", offs[n], ohdr[n], 0, 0)
    snod_addr = put(bytes(snod))
    btree = put(b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", 1, UNDEF, UNDEF) +
                struct.pack("<QQQ", 0, snod_addr, offs[names[-1]]))
    root = put(_ohdr([_msg(0x11, struct.pack("<QQ", btree, heap_addr))]))
    sb = b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, len(out), UNDEF)
    sb += struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", btree, heap_addr)
    out[:96] = sb
    with open(path, "wb") as f:
        f.write(bytes(out))
