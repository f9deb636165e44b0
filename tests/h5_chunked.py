"""Test infrastructure: HDF5 files with a CHUNKED dataset, written from the HDF5 file-format
specification independently of the library's reader, with the chunk payloads compressed by
Python's zlib (the same stream format HDF5's deflate filter produces).

The file skeleton (superblock, root group, the datatype message) comes from the library's own
writer, for a one-element placeholder of the dataset's type. A new version-1 object header is
appended with a version-3 chunked layout message (rank + 1 chunk dimensions, the last one the
element size), a filter pipeline message and a version-1 B-tree of raw-data chunks (node type
1: keys of chunk size, filter mask and rank + 1 offsets), and the root group's symbol table entry
is pointed at it.
"""
import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
FILTER_IDS = {"deflate": 1, "shuffle": 2, "fletcher32": 3}


def _msg(mtype, body, flags=0):
    body = bytes(body)
    pad = (-len(body)) % 8
    return struct.pack("<HHB3x", mtype, len(body) + pad, flags) + body + b"\0" * pad


def _header_messages(b, addr):
    """(type, body) of a version-1 object header without continuation blocks."""
    assert b[addr] == 1
    nmsg, size = struct.unpack_from("<H", b, addr + 2)[0], struct.unpack_from("<I", b, addr + 8)[0]
    p, end, out = addr + 16, addr + 16 + size, []
    while p + 8 <= end and len(out) < nmsg:
        t, s = struct.unpack_from("<HH", b, p)
        out.append((t, bytes(b[p + 8:p + 8 + s])))
        p += 8 + s
    return out


def _shuffle(raw, esz):
    a = np.frombuffer(raw, np.uint8)
    n = len(a) // esz
    head = a[:n * esz].reshape(n, esz).T.reshape(-1)
    return head.tobytes() + a[n * esz:].tobytes()


def _pipeline_message(filters, esz, level, version):
    body = bytearray([version, len(filters)])
    if version == 1:
        body += b"\0" * 6
    for f in filters:
        fid = FILTER_IDS[f]
        cd = {"deflate": [level], "shuffle": [esz], "fletcher32": []}[f]
        name = (f + "\0").encode()
        if version == 1:
            name += b"\0" * ((-len(name)) % 8)
            body += struct.pack("<HHHH", fid, len(name), 0, len(cd)) + name
        else:                       # version 2: no name field below id 256
            body += struct.pack("<HHH", fid, 0, len(cd))
        body += b"".join(struct.pack("<I", v) for v in cd)
        if version == 1 and len(cd) % 2:
            body += b"\0" * 4
    return _msg(0x000B, body)


def _deflate(data, level, strategy, wbits):
    c = zlib.compressobj(level, zlib.DEFLATED, wbits, 9, strategy)
    return c.compress(data) + c.flush()


def write_chunked(path, name, array, chunks, filters=("shuffle", "deflate"), level=6,
                  pipeline_version=1, leaf_entries=8, skip_chunks=(), raw_chunks=(),
                  strategy=zlib.Z_DEFAULT_STRATEGY, wbits=15):
    """Writes `array` as the chunked dataset `name` of a new HDF5 file.

    chunks: chunk shape; filters: applied in this order on write; skip_chunks: chunk grid
    indices left unwritten (they read as zeros); raw_chunks: chunk grid indices stored with
    every filter skipped (filter mask all ones); leaf_entries: chunks per B-tree leaf (more
    chunks than that make a two-level tree); strategy, wbits: zlib's deflate strategy and
    window (fixed or dynamic Huffman blocks, run-length matches, short windows)."""
    from spinwalk_gb300 import _lib
    array = np.ascontiguousarray(array)
    rank, esz = array.ndim, array.dtype.itemsize
    _lib.h5_write(path, {name: np.zeros((1,), array.dtype)})
    b = bytearray(open(path, "rb").read())
    snod = b.find(b"SNOD")
    old_ohdr = struct.unpack_from("<Q", b, snod + 16)[0]
    dtype_body = next(body for t, body in _header_messages(b, old_ohdr) if t == 0x0003)

    def append(blob):
        while len(b) % 8:
            b.append(0)
        at = len(b)
        b.extend(blob)
        return at

    grid = [-(-d // c) for d, c in zip(array.shape, chunks)]
    entries = []                                        # (key bytes, chunk address)
    for idx in np.ndindex(*grid):
        if idx in skip_chunks:
            continue
        lo = [i * c for i, c in zip(idx, chunks)]
        block = np.zeros(chunks, array.dtype)
        sl = tuple(slice(l, min(l + c, d)) for l, c, d in zip(lo, chunks, array.shape))
        block[tuple(slice(0, s.stop - s.start) for s in sl)] = array[sl]
        data = block.tobytes()
        mask = 0
        if idx in raw_chunks:
            mask = (1 << len(filters)) - 1
        else:
            for f in filters:
                if f == "shuffle":
                    data = _shuffle(data, esz)
                elif f == "deflate":
                    data = _deflate(data, level, strategy, wbits)
                else:               # a 4-byte checksum trailer (the reader drops it)
                    data = data + struct.pack("<I", zlib.crc32(data))
        addr = append(data)
        key = struct.pack("<II", len(data), mask) + b"".join(
            struct.pack("<Q", v) for v in lo + [0])
        entries.append((key, addr))
    end_key = struct.pack("<II", 0, 0) + b"".join(struct.pack("<Q", v) for v in
                                                   list(array.shape) + [0])

    def node(level, items, last_key):
        blob = b"TREE" + struct.pack("<BBHQQ", 1, level, len(items), UNDEF, UNDEF)
        for key, child in items:
            blob += key + struct.pack("<Q", child)
        return append(blob + last_key)

    if not entries:
        btree = UNDEF
    elif len(entries) <= leaf_entries:
        btree = node(0, entries, end_key)
    else:
        leaves = []
        for k in range(0, len(entries), leaf_entries):
            part = entries[k:k + leaf_entries]
            nxt = entries[k + leaf_entries][0] if k + leaf_entries < len(entries) else end_key
            leaves.append((part[0][0], node(0, part, nxt)))
        btree = node(1, leaves, end_key)

    space = bytes([1, rank, 0, 0, 0, 0, 0, 0]) + b"".join(struct.pack("<Q", d) for d in array.shape)
    layout = bytes([3, 2, rank + 1]) + struct.pack("<Q", btree) + b"".join(
        struct.pack("<I", c) for c in list(chunks) + [esz])
    msgs = _msg(0x0001, space) + _msg(0x0003, dtype_body, 1) + _msg(0x0008, layout)
    nmsg = 3
    if filters:
        msgs += _pipeline_message(filters, esz, level, pipeline_version)
        nmsg += 1
    ohdr = append(struct.pack("<BBHII4x", 1, 0, nmsg, 1, len(msgs)) + msgs)
    struct.pack_into("<Q", b, snod + 16, ohdr)
    struct.pack_into("<Q", b, 40, len(b))               # end-of-file address
    open(path, "wb").write(bytes(b))
